// Matrix-free Q4 hexahedral Laplacian action (sum factorisation).
//
// The operator of the matrix-free Poisson demo (cpp/demo/poisson_matrix_free/
// main.cpp:201-222) for Lagrange Q4 on a structured hexahedral mesh with
// trilinear geometry: Gauss-Lobatto-Legendre nodes, Gauss-Legendre 5^3
// quadrature, nodes numbered lexicographically on the (4n+1)^3 lattice.
// y = A u on interior nodes (boundary entries of u read as 0) and y = u on
// boundary nodes: the homogeneous Dirichlet rows set to the identity.
#pragma once

#include "common.cuh"

using dfx_q4_mesh_s = dfx_q4_mesh;

namespace dfx
{
// Uploads the 1D basis tables to the current device (once per device).
// Must run outside stream capture; q4_apply calls it too.
int q4_prepare();

// y = A u with T = float or double (u, y of that type). Launches a memset
// and 8 colour kernels on `s`. When `skip` is given and *skip != 0 at run
// time, the colour kernels return at once (a solver that has converged
// inside a replayed graph).
template <typename T>
int q4_apply(const dfx_q4_mesh_s& m, const T* u, T* y, cudaStream_t s,
             const int32_t* skip = nullptr);

// y = A u in FP32 with the basis contractions on the tensor cores
// (tcgen05, TF32 with a three-term split); same launches as q4_apply<float>.
int q4_apply_tc(const dfx_q4_mesh_s& m, const float* u, float* y, cudaStream_t s,
                const int32_t* skip = nullptr);

// DFX_ERR_TIMEOUT (and the flag cleared) when a tensor-core kernel gave up
// waiting for an MMA since the last check; synchronous.
int q4_tc_check();

inline int64_t q4_ndofs(const dfx_q4_mesh_s& m)
{
  return (4 * (int64_t)m.nx + 1) * (4 * (int64_t)m.ny + 1) * (4 * (int64_t)m.nz + 1);
}
} // namespace dfx
