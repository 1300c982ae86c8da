// A caller's own element kernels compiled around the library's cell loops
// (include/dfx_cell_kernel.cuh): P1 Poisson a(u,v) = \int kappa grad u .
// grad v with kappa a per-cell coefficient, and a P1 load L(v) = \int c0 v
// with c0 a constant. Built by the tests with nvcc into a shared object and
// compared with the library's built-in forms.
#include "dfx_cell_kernel.cuh"

namespace
{
// Gradients of the 4 barycentrics of an affine tetrahedron and |det J|.
__device__ double p1_gradients(const double* X, double g[4][3])
{
  double J[3][3];
  for (int d = 0; d < 3; ++d)
    for (int k = 0; k < 3; ++k)
      J[d][k] = X[3 * (k + 1) + d] - X[d];
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double inv[3][3] = {
      {c00 / det, (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det,
       (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det},
      {c01 / det, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det,
       (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det},
      {c02 / det, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det,
       (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det}};
  for (int d = 0; d < 3; ++d)
  {
    g[1][d] = inv[0][d];
    g[2][d] = inv[1][d];
    g[3][d] = inv[2][d];
    g[0][d] = -(g[1][d] + g[2][d] + g[3][d]);
  }
  return det < 0 ? -det : det;
}

struct P1Poisson
{
  __device__ void operator()(double* A, const double* w, const double*, const double* X,
                             int) const
  {
    double g[4][3];
    const double vol = p1_gradients(X, g) / 6.0;
    const double kappa = w ? w[0] : 1.0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        A[4 * i + j] = kappa * vol * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
  }
};

struct P1Load
{
  __device__ void operator()(double* b, const double*, const double* c, const double* X,
                             int) const
  {
    double g[4][3];
    const double vol = p1_gradients(X, g) / 6.0;
    for (int i = 0; i < 4; ++i)
      b[i] = c[0] * vol / 4.0;
  }
};
} // namespace

extern "C" int user_assemble_p1_poisson(int32_t num_cells, const int32_t* x_dofmap,
                                        const double* x, const int32_t* dofmap,
                                        const double* kappa, const int8_t* bc, const dfx_csr* A,
                                        int* status, void* stream)
{
  return (int)dfx_user::launch_assemble_matrix<4, 1>(P1Poisson{}, num_cells, x_dofmap, x,
                                                      dofmap, kappa, 1, nullptr, bc, *A, status,
                                                      (cudaStream_t)stream);
}

extern "C" int user_assemble_p1_load(int32_t num_cells, const int32_t* x_dofmap, const double* x,
                                     const int32_t* dofmap, const double* c, double* b,
                                     void* stream)
{
  return (int)dfx_user::launch_assemble_vector<4, 1>(P1Load{}, num_cells, x_dofmap, x, dofmap,
                                                      nullptr, 0, c, b, (cudaStream_t)stream);
}
