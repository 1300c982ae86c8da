/* Device cell loops around a caller's own element kernel.
 *
 * The reference takes each cell's element tensor from a kernel called
 * through a function pointer with the ABI of fem/kernel.h:18-27,
 *   void(T* A, const T* w, const T* c, const U* coordinate_dofs,
 *        const int* entity_local_index, const uint8_t* perm, void* data),
 * once per cell (fem/assemble_matrix_impl.h:92-200,
 * fem/assemble_vector_impl.h:75-116). A device function pointer would cost
 * an indirect call per cell and cannot cross the library's module, so the
 * GPU counterpart is a template: the caller compiles these loops with nvcc
 * around an element functor of the same shape,
 *
 *   struct MyKernel {
 *     __device__ void operator()(double* A, const double* w, const double* c,
 *                                const double* coordinate_dofs, int cell) const;
 *   };
 *
 * where A is the (ND*BS) x (ND*BS) row-major element matrix (or the ND*BS
 * element vector), w the cell's packed coefficients (cstride values), c the
 * form's constants and coordinate_dofs the cell's 4 vertices (3 doubles
 * each) -- the reference's arguments for an affine tetrahedron, whose
 * entity_local_index and permutation data are not used by cell integrals.
 * The loops are those of the built-in forms: one thread per cell, rows and
 * columns of constrained dofs (bc, indexed by BS * node + component) zeroed,
 * FP64 atomic scatter into the CSR values found by binary search in each
 * row ("Entry not in sparsity" sets *status to DFX_ERR_NOT_IN_SPARSITY), and
 * accumulate semantics (nothing is zeroed first). Only this header and
 * dfx_gpu.h are needed; no symbol of libdfxgpu.so is used.
 */
#ifndef DFX_CELL_KERNEL_CUH
#define DFX_CELL_KERNEL_CUH

#include "dfx_gpu.h"

#include <cstdint>
#include <cuda_runtime.h>

namespace dfx_user
{
/* Cell vertex coordinates in the reference's coordinate_dofs layout. */
__device__ inline void cell_coordinates(const int32_t* x_dofmap, const double* x, int32_t c,
                                        double* coords)
{
  for (int v = 0; v < 4; ++v)
  {
    const int64_t node = x_dofmap[4 * (int64_t)c + v];
    for (int k = 0; k < 3; ++k)
      coords[3 * v + k] = x[3 * node + k];
  }
}

/* Position of column `col` in row [b, e) of a sorted CSR (e if absent). */
__device__ inline int64_t csr_find(const int32_t* cols, int64_t b, int64_t e, int32_t col)
{
  while (b < e)
  {
    const int64_t m = b + (e - b) / 2;
    if (cols[m] < col)
      b = m + 1;
    else
      e = m;
  }
  return b;
}

template <int ND, int BS, class Kernel>
__global__ void assemble_matrix_cells(Kernel kernel, int32_t num_cells, const int32_t* x_dofmap,
                                      const double* x, const int32_t* dofmap, const double* w,
                                      int32_t cstride, const double* c, const int8_t* bc,
                                      const int64_t* row_ptr, const int32_t* cols, double* vals,
                                      int* status)
{
  constexpr int N = ND * BS;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= num_cells)
    return;
  double coords[12];
  cell_coordinates(x_dofmap, x, (int32_t)cell, coords);
  double A[N * N];
  for (int i = 0; i < N * N; ++i)
    A[i] = 0.0;
  kernel(A, w ? w + cell * cstride : nullptr, c, coords, (int)cell);
  const int32_t* dofs = dofmap + cell * ND;
  for (int i = 0; i < ND; ++i)
  {
    const int32_t row = dofs[i];
    const int64_t rb = row_ptr[row], re = row_ptr[row + 1];
    for (int j = 0; j < ND; ++j)
    {
      const int32_t col = dofs[j];
      const int64_t p = csr_find(cols, rb, re, col);
      if (p >= re || cols[p] != col)
      {
        atomicExch(status, (int)DFX_ERR_NOT_IN_SPARSITY);
        continue;
      }
      for (int a = 0; a < BS; ++a)
      {
        if (bc && bc[BS * row + a])
          continue;
        for (int b = 0; b < BS; ++b)
        {
          if (bc && bc[BS * col + b])
            continue;
          atomicAdd(vals + p * BS * BS + a * BS + b, A[(BS * i + a) * N + BS * j + b]);
        }
      }
    }
  }
}

template <int ND, int BS, class Kernel>
__global__ void assemble_vector_cells(Kernel kernel, int32_t num_cells, const int32_t* x_dofmap,
                                      const double* x, const int32_t* dofmap, const double* w,
                                      int32_t cstride, const double* c, double* b)
{
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= num_cells)
    return;
  double coords[12];
  cell_coordinates(x_dofmap, x, (int32_t)cell, coords);
  double be[ND * BS];
  for (int i = 0; i < ND * BS; ++i)
    be[i] = 0.0;
  kernel(be, w ? w + cell * cstride : nullptr, c, coords, (int)cell);
  const int32_t* dofs = dofmap + cell * ND;
  for (int i = 0; i < ND; ++i)
    for (int k = 0; k < BS; ++k)
      atomicAdd(b + BS * (int64_t)dofs[i] + k, be[BS * i + k]);
}

/* Launch the matrix loop on `stream`; returns the CUDA launch status. The
 * caller reads *status (device memory, zeroed by the caller) afterwards. */
template <int ND, int BS, class Kernel>
cudaError_t launch_assemble_matrix(const Kernel& kernel, int32_t num_cells,
                                   const int32_t* x_dofmap, const double* x,
                                   const int32_t* dofmap, const double* w, int32_t cstride,
                                   const double* c, const int8_t* bc, const dfx_csr& A,
                                   int* status, cudaStream_t stream)
{
  if (num_cells <= 0)
    return cudaSuccess;
  const unsigned grid = (unsigned)((num_cells + 127) / 128);
  assemble_matrix_cells<ND, BS, Kernel><<<grid, 128, 0, stream>>>(
      kernel, num_cells, x_dofmap, x, dofmap, w, cstride, c, bc, A.row_ptr, A.cols,
      (double*)A.vals, status);
  return cudaGetLastError();
}

template <int ND, int BS, class Kernel>
cudaError_t launch_assemble_vector(const Kernel& kernel, int32_t num_cells,
                                   const int32_t* x_dofmap, const double* x,
                                   const int32_t* dofmap, const double* w, int32_t cstride,
                                   const double* c, double* b, cudaStream_t stream)
{
  if (num_cells <= 0)
    return cudaSuccess;
  const unsigned grid = (unsigned)((num_cells + 127) / 128);
  assemble_vector_cells<ND, BS, Kernel><<<grid, 128, 0, stream>>>(
      kernel, num_cells, x_dofmap, x, dofmap, w, cstride, c, b);
  return cudaGetLastError();
}
} // namespace dfx_user

#endif /* DFX_CELL_KERNEL_CUH */
