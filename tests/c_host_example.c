/* A plain C host of libdfxgpu: builds a 4^3 x 6 box mesh with RCM order, a
 * P2 dofmap, its sparsity pattern and exterior facets through the C ABI,
 * reads a timing back, and checks an error path. Host functions only, so
 * it runs without a GPU. Prints one line of counts. */
#include "dfx_gpu.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int fail(const char* what)
{
  fprintf(stderr, "%s: %s\n", what, dfx_last_error());
  return 1;
}

int main(void)
{
  const int n = 4, nc = 6 * n * n * n, nv = (n + 1) * (n + 1) * (n + 1);
  const double p0[3] = {0.0, 0.0, 0.0}, p1[3] = {1.0, 1.0, 1.0};
  int32_t* cells = malloc(sizeof(int32_t) * 4 * nc);
  double* x = malloc(sizeof(double) * 3 * nv);
  int32_t* dofmap = malloc(sizeof(int32_t) * 10 * nc);
  int32_t* facets = malloc(sizeof(int32_t) * 8 * nc);
  int32_t nodes = 0, nf = 0, ni = 0, reps = 0;
  int64_t nnz = 0;
  double seconds = 0.0;
  if (!cells || !x || !dofmap || !facets)
    return 2;
  if (dfx_mesh_create_box_tet(n, n, n, p0, p1, 1, cells, x) != DFX_OK)
    return fail("mesh");
  if (dfx_dofmap_create_tet(nc, cells, 2, dofmap, &nodes) != DFX_OK)
    return fail("dofmap");
  int64_t* row_ptr = malloc(sizeof(int64_t) * (nodes + 1));
  if (!row_ptr || dfx_sparsity_create(nodes, nc, 10, dofmap, row_ptr, NULL, &nnz) != DFX_OK)
    return fail("sparsity count");
  int32_t* cols = malloc(sizeof(int32_t) * (size_t)nnz);
  if (!cols || dfx_sparsity_create(nodes, nc, 10, dofmap, row_ptr, cols, &nnz) != DFX_OK)
    return fail("sparsity fill");
  if (dfx_exterior_facets_tet(nc, cells, facets, &nf) != DFX_OK)
    return fail("facets");
  /* the facets buffer is reused: interior facets need as much room */
  if (dfx_interior_facets_tet(nc, cells, facets, &ni) != DFX_OK)
    return fail("interior facets");
  if (dfx_timing("Build BoxMesh (tetrahedra)", &reps, &seconds) != DFX_OK)
    return fail("timing");
  /* an invalid box is refused with the reference's message */
  if (dfx_mesh_create_box_tet(0, 1, 1, p0, p1, 1, cells, x) != DFX_ERR_INVALID ||
      strcmp(dfx_last_error(), "At least one cell is required.") != 0)
    return 3;
  printf("abi %d cells %d nodes %d nnz %lld facets %d interior %d mesh_reps %d\n",
         dfx_abi_version(), nc, nodes, (long long)nnz, nf, ni, reps);
  free(cols);
  free(row_ptr);
  free(facets);
  free(dofmap);
  free(x);
  free(cells);
  return 0;
}
