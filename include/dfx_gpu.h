/* dfx_gpu.h -- C ABI of the GB300 (sm_103a) FEM assembly + CG hot path.
 *
 * libdfxgpu.so replaces, behind DOLFINx's own C++ API, the cell loops of
 * fem::assemble_matrix / fem::assemble_vector, fem::apply_lifting,
 * DirichletBC::set, set_diagonal, MatrixCSR::mult and the CG iteration of
 * the matrix-free Poisson demo. Every entry point takes plain pointers and
 * sizes and returns an int status (DFX_OK == 0); dfx_last_error() gives the
 * message of the last failure on the calling thread. Pointers named d_*
 * are device pointers; `stream` is a cudaStream_t (NULL = default stream).
 * Arrays are caller-owned; nothing is freed by the library.
 *
 * Paths cited below are relative to the DOLFINx source tree.
 */
#ifndef DFX_GPU_H
#define DFX_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum dfx_status
{
  DFX_OK = 0,
  DFX_ERR_INVALID = 1,           /* bad argument or size mismatch */
  DFX_ERR_CUDA = 2,              /* CUDA runtime error */
  DFX_ERR_NOT_IN_SPARSITY = 3,   /* "Entry not in sparsity" (la/matrix_csr_impl.h:93-94) */
  DFX_ERR_NOT_CONVERGED = 4,     /* CG hit its iteration cap */
  DFX_ERR_TIMEOUT = 5,           /* a bounded device wait gave up */
  DFX_ERR_NO_MEMORY = 6,         /* workspace too small / HBM budget exceeded */
  DFX_ERR_BREAKDOWN = 7,         /* CG breakdown (p.Ap <= 0 or NaN) */
  DFX_ERR_UNSUPPORTED = 8
};

/* Message of the last failing call on this thread ("" if none). */
const char* dfx_last_error(void);
int dfx_abi_version(void);

/* ---------------------------------------------------------------- types */
enum dfx_form_kind
{
  /* a(u,v) = \int kappa grad u . grad v + k2 u v dx, Lagrange P1/P2 tets */
  DFX_FORM_POISSON = 0,
  /* a(u,v) = \int 2 mu eps(u):eps(v) + lambda div u div v, vector P2, bs 3,
     mu, lambda from a per-cell Young's modulus E (kappa) and nu */
  DFX_FORM_ELASTICITY = 1,
  /* L(v) = \int f v dx, f a P1 coefficient on the geometry nodes (f == NULL:
     f = f_const[0]) */
  DFX_FORM_SOURCE = 2,
  /* L(v) = \int f . v dx, f = f_const (vector P2, bs 3) */
  DFX_FORM_BODYFORCE = 3,
  /* a(u,v) = \int_F alpha u v ds over exterior facets (Robin term), alpha =
     kappa of the facet's cell or kappa_const; scalar P1/P2 */
  DFX_FORM_FACET_MASS = 4,
  /* a(u,v) = \int_F gamma |F| [grad u . n][grad v . n] dS over interior
     facets (continuous interior penalty), gamma the average of the two
     cells' kappa (or kappa_const); scalar P1/P2 */
  DFX_FORM_FACET_JUMP = 5
};

enum dfx_assembly_mode
{
  DFX_MODE_ATOMIC = 0,   /* FP64 atomic scatter, one launch */
  DFX_MODE_COLOURED = 1  /* cells grouped by colour, plain adds: deterministic */
};

enum dfx_dtype
{
  DFX_F64 = 0,
  DFX_F32 = 1,
  /* Operators only: an FP64 value carried as two FP32 words, hi = fl32(v)
   * and lo = fl32(v - hi), multiplied on the FP32 pipe with error-free
   * transformations (FP64-equivalent products; vectors stay FP64). */
  DFX_F32X2 = 2
};

/* A form on a tetrahedral mesh, all arrays on the device.
 * Replaces fem::Form + the FFCx kernel of its cell integral
 * (fem/Form.h:116-668, fem/kernel.h:18-27): the element kernel is chosen
 * by `kind`, the coefficients are packed per cell (fem/pack.h:77-176). */
typedef struct dfx_form
{
  int32_t kind;            /* dfx_form_kind */
  int32_t degree;          /* 1 or 2 (elasticity/body force: 2) */
  int32_t num_cells;
  int32_t num_nodes;       /* rows of x */
  const int32_t* x_dofmap; /* (num_cells, 4) geometry dofmap */
  const double* x;         /* (num_nodes, 3) coordinates */
  const int32_t* dofmap;   /* (num_cells, ndofs) node (block) indices */
  const double* kappa;     /* per-cell kappa / E, or NULL -> kappa_const */
  double kappa_const;
  double k2;               /* Helmholtz mass coefficient (scalar bilinear) */
  double nu;               /* Poisson ratio (elasticity) */
  const double* f;         /* P1 source values per geometry node, or NULL */
  double f_const[3];
} dfx_form;

/* A CSR matrix with square bs x bs blocks on the device, the storage of
 * la::MatrixCSR (la/MatrixCSR.h:67-70): row_ptr int64 (nrows+1), cols
 * int32 (nnz, sorted per row), vals nnz*bs*bs, blocks row-major. */
typedef struct dfx_csr
{
  int32_t nrows;  /* block rows */
  int32_t ncols;  /* block columns */
  int32_t bs;     /* 1 or 3 */
  int32_t dtype;  /* dfx_dtype of vals */
  int64_t nnz;    /* blocks */
  const int64_t* row_ptr;
  const int32_t* cols;
  void* vals;
} dfx_csr;

/* ---------------------------------------------------------- host set-up
 * One-time structure built on the host CPU. Results are bit-identical to
 * DOLFINx on one rank. */

/* mesh::create_box(tetrahedron) with the default RCM cell reordering
 * (mesh/generation.h:104-134, 380-426; mesh/utils.h:232-310;
 * graph/ordering.cpp:148-170). cells: (6 nx ny nz, 4) geometry node
 * indices; x: ((nx+1)(ny+1)(nz+1), 3). reorder = 0 keeps build order. */
int dfx_mesh_create_box_tet(int32_t nx, int32_t ny, int32_t nz, const double* p0,
                            const double* p1, int32_t reorder, int32_t* cells,
                            double* x);

/* mesh::build_local_dual_graph for one tetrahedral cell type, serial path
 * (mesh/graphbuild.cpp:566-905): cells joined by a facet. offsets
 * (num_cells+1); adj (capacity 4*num_cells) lists, for each cell, the other
 * cells of each of its facets in sorted-facet order, as the reference's
 * edge-by-edge fill gives. Host function, threaded. */
int dfx_mesh_dual_graph_tet(int32_t num_cells, const int32_t* cells, int32_t num_vertices,
                            int32_t* offsets, int32_t* adj);

/* graph::reorder_rcm (graph/ordering.cpp:148-170): the reverse
 * Cuthill-McKee permutation of a graph (offsets n+1, adjacency), perm[old]
 * = new, with the reference's George-Liu pseudo-peripheral root and degree
 * tie order. The graph is taken as given (symmetric, as a dual graph is).
 * Host function; large graphs run level by level on threads. */
int dfx_graph_reorder_rcm(int32_t n, const int32_t* offsets, const int32_t* adj,
                          int32_t* perm);

/* The same three set-up steps on the device, bit-identical to the host
 * functions above (the same definitions, see mesh_device.cu):
 *
 * dfx_mesh_create_box_tet_device: d_cells (num_cells x 4 int32, 16-byte
 * aligned) and d_x (num_vertices x 3 doubles) in device memory, the mesh
 * of dfx_mesh_create_box_tet. Coordinates are p0 + i * (p1 - p0) / n
 * without a fused multiply-add, as the reference's expression compiles on
 * x86-64 (mesh/generation.h:332-377).
 *
 * dfx_mesh_dual_graph_tet_device: device offsets (num_cells + 1) and
 * adjacency (capacity 4 num_cells) of dfx_mesh_dual_graph_tet. Returns
 * DFX_ERR_UNSUPPORTED when a facet is shared by more than two cells (the
 * host function applies).
 *
 * dfx_graph_reorder_rcm_device: device offsets/adjacency in, device perm
 * (perm[old] = new) out, as dfx_graph_reorder_rcm. Returns
 * DFX_ERR_UNSUPPORTED for a node of degree above 16 (the degree sort then
 * follows libstdc++'s introsort, which the device does not restate).
 *
 * Each takes a device workspace of its *_workspace_bytes (256-byte
 * aligned), runs on `stream` and synchronises it before returning. */
size_t dfx_mesh_create_box_tet_device_workspace_bytes(int32_t nx, int32_t ny, int32_t nz,
                                                      int32_t reorder);
int dfx_mesh_create_box_tet_device(int32_t nx, int32_t ny, int32_t nz, const double* p0,
                                   const double* p1, int32_t reorder, int32_t* d_cells,
                                   double* d_x, void* d_work, size_t work_bytes, void* stream);
size_t dfx_mesh_dual_graph_tet_device_workspace_bytes(int32_t num_cells, int32_t num_vertices);
int dfx_mesh_dual_graph_tet_device(int32_t num_cells, const int32_t* d_cells,
                                   int32_t num_vertices, int32_t* d_offsets, int32_t* d_adj,
                                   void* d_work, size_t work_bytes, void* stream);
size_t dfx_graph_reorder_rcm_device_workspace_bytes(int32_t n);
int dfx_graph_reorder_rcm_device(int32_t n, const int32_t* d_offsets, const int32_t* d_adj,
                                 int32_t* d_perm, void* d_work, size_t work_bytes, void* stream);

/* fem::create_dofmap for Lagrange P1/P2 on tetrahedra
 * (fem/utils.cpp:32-76, fem/dofmapbuilder.cpp:153-710). dofmap:
 * (num_cells, 4 or 10). Returns the number of dof nodes in *num_nodes. */
int dfx_dofmap_create_tet(int32_t num_cells, const int32_t* cells, int32_t degree,
                          int32_t* dofmap, int32_t* num_nodes);

/* The same dofmap built on the device (fem::create_dofmap numbering:
 * first appearance in the cell loop, fem/dofmapbuilder.cpp:440-474):
 * bit-identical to dfx_dofmap_create_tet. d_cells 16-byte aligned, vertex
 * indices in [0, num_vertices); d_dofmap (num_cells x 4 or 10). Workspace
 * of dfx_dofmap_device_workspace_bytes, 256-byte aligned. Returns
 * DFX_ERR_UNSUPPORTED when the edge table overflows (meshes with more than
 * ~2.5 edges per cell): the host builder then applies. Synchronises. */
size_t dfx_dofmap_device_workspace_bytes(int32_t num_cells, int32_t num_vertices, int32_t degree);
int dfx_dofmap_create_tet_device(int32_t num_cells, const int32_t* d_cells, int32_t num_vertices,
                                 int32_t degree, int32_t* d_dofmap, int32_t* num_nodes,
                                 void* d_work, size_t work_bytes, void* stream);

/* fem::create_sparsity_pattern + SparsityPattern::finalize
 * (fem/utils.h:197-314, la/SparsityPattern.cpp:264-491) for a cell integral
 * with the same dofmap on both sides. Two-phase: call with cols == NULL to
 * get *nnz and row_ptr (nrows+1), then again with cols (nnz). */
int dfx_sparsity_create(int32_t nrows, int32_t num_cells, int32_t ndofs,
                        const int32_t* dofmap, int64_t* row_ptr, int32_t* cols,
                        int64_t* nnz);

/* The same pattern built on the device from a device dofmap (same
 * reference functions): d_row_ptr and d_cols equal dfx_sparsity_create's
 * bit for bit. Two-phase: with d_cols == NULL it writes d_row_ptr
 * (nrows+1) and *nnz; then call again with d_cols (nnz) and the d_row_ptr
 * of the first call. d_work: dfx_sparsity_device_workspace_bytes() bytes,
 * 256-byte aligned. A row whose cells hold more than 1024 dofs in total
 * returns DFX_ERR_UNSUPPORTED (use the host builder). Synchronises
 * `stream`. */
size_t dfx_sparsity_device_workspace_bytes(int32_t nrows, int32_t num_cells,
                                           int32_t ndofs);
int dfx_sparsity_create_device(int32_t nrows, int32_t num_cells, int32_t ndofs,
                               const int32_t* d_dofmap, int64_t* d_row_ptr,
                               int32_t* d_cols, int64_t* nnz, void* d_work,
                               size_t work_bytes, void* stream);

/* FunctionSpace::tabulate_dof_coordinates (fem/FunctionSpace.h:218-330) for
 * Lagrange P1/P2 on affine tetrahedra: X (num_nodes, 3) receives each dof
 * node's point, the cell vertices and the edge midpoints 0.5 (a + b) in
 * Basix edge order. Nodes that no cell holds are not written (the caller
 * zeroes X, as the reference does). Every index is checked before anything
 * is written. Host function, threaded. */
int dfx_tabulate_dof_coordinates_tet(int32_t num_cells, const int32_t* cells,
                                     int32_t num_vertices, const double* x,
                                     const int32_t* dofmap, int32_t degree,
                                     int32_t num_nodes, double* X);

/* Greedy cell colouring for DFX_MODE_COLOURED: no two cells of one colour
 * share a dof. order: (num_cells) cells grouped by colour, offsets:
 * (max_colours+1). Returns the colour count in *num_colours. */
int dfx_colour_cells(int32_t num_cells, int32_t ndofs, const int32_t* dofmap,
                     int32_t num_nodes, int32_t* order, int32_t* offsets,
                     int32_t max_colours, int32_t* num_colours);

/* ------------------------------------------------------------- assembly */

/* Bytes of the cell -> CSR slot map (one byte per element entry). */
size_t dfx_slot_map_bytes(const dfx_form* a);

/* Cell -> CSR slot map, built once from the sparsity pattern: for cell c
 * and local dofs (i, j), d_map[(c*nd + i)*nd + j] is the position of
 * dofmap[c,j] within row dofmap[c,i]. Fails with DFX_ERR_NOT_IN_SPARSITY
 * when an entry is missing, DFX_ERR_UNSUPPORTED when a row is longer
 * than 255. Replaces the per-entry std::lower_bound of insert_csr
 * (la/matrix_csr_impl.h:86-94). */
int dfx_slot_map_create(const dfx_form* a, const dfx_csr* A, uint8_t* d_map,
                        void* stream);

/* fem::assemble_matrix (fem/assembler.h:513-602;
 * fem/assemble_matrix_impl.h:92-200): A += sum_cells Ae, rows and
 * columns of constrained dofs (d_bc[bs*node+k] != 0) zeroed in Ae.
 * d_map from dfx_slot_map_create, or NULL to search the row.
 * DFX_MODE_COLOURED needs d_order/colour_offsets (host array) from
 * dfx_colour_cells (uploaded order). A is accumulated, not zeroed. */
int dfx_assemble_matrix(const dfx_form* a, const dfx_csr* A, const uint8_t* d_map,
                        const int8_t* d_bc, int32_t mode, const int32_t* d_order,
                        const int32_t* colour_offsets, int32_t num_colours,
                        void* stream);

/* fem::assemble_vector (fem/assembler.h:229-257;
 * fem/assemble_vector_impl.h:75-116): b += sum_cells be. */
int dfx_assemble_vector(const dfx_form* L, double* d_b, int32_t mode,
                        const int32_t* d_order, const int32_t* colour_offsets,
                        int32_t num_colours, void* stream);

/* fem::apply_lifting for one bilinear form (fem/assembler.h:341-421;
 * fem/assemble_vector_impl.h:361-414): for cells with a constrained
 * column, b[r] -= Ae[r,c] * alpha * (g[c] - x0[c]). d_x0 may be NULL. */
int dfx_apply_lifting(const dfx_form* a, double* d_b, const int8_t* d_bc,
                      const double* d_g, const double* d_x0, double alpha,
                      int32_t mode, const int32_t* d_order,
                      const int32_t* colour_offsets, int32_t num_colours,
                      void* stream);

/* DirichletBC::set (fem/DirichletBC.h:495-578): x[dofs[i]] =
 * alpha * (g - x0) with g = d_g[dofs[i]] (or g_const when d_g is NULL);
 * dofs >= n are skipped. */
int dfx_set_bc(double* d_x, int64_t n, const int32_t* d_dofs, int32_t ndofs,
               const double* d_g, double g_const, const double* d_x0,
               double alpha, void* stream);

/* set_diagonal (fem/assembler.h:644-686) through MatrixCSR::set:
 * A[d, d] = diagonal for each constrained scalar dof d. */
int dfx_set_diagonal(const dfx_csr* A, const int32_t* d_dofs, int32_t ndofs,
                     double diagonal, void* stream);

/* --------------------------------------------------------- linear algebra */

/* MatrixCSR::mult (la/MatrixCSR.h:877-946; la/matrix_csr_impl.h:259-286):
 * y = beta*y + A x, beta in {0, 1} (1 = the reference's y += A x).
 * dtype of x/y equals A->dtype. */
int dfx_spmv(const dfx_csr* A, const void* d_x, void* d_y, double beta,
             void* stream);

/* Cast of MatrixCSR values to float (la/MatrixCSR.h:223-237). */
int dfx_csr_values_to_f32(const dfx_csr* A, float* d_vals32, void* stream);

/* The scalar CSR of a bs x bs block CSR: row bs*I + k0 holds the entries
 * (bs*J + k1) of every block J of block row I, in ascending column order
 * (la/MatrixCSR.h:56-66 block layout). row_ptr: nrows*bs + 1 entries;
 * cols, vals: nnz*bs*bs. d_cols == NULL refreshes the values only. Lets
 * the scalar solvers (sliced-ELL operators, refinement) take vector-valued
 * problems such as elasticity. */
int dfx_csr_expand_blocks(const dfx_csr* A, int64_t* d_row_ptr, int32_t* d_cols,
                          double* d_vals, void* stream);

/* d_dinv[i] = 1 / A_ii (Jacobi), scalar rows of a bs-blocked matrix. */
int dfx_jacobi_inverse_diagonal(const dfx_csr* A, double* d_dinv, void* stream);

/* la::inner_product (la/Vector.h:434-460), deterministic two-stage
 * reduction; the result is written to *result (host). */
size_t dfx_inner_product_workspace_bytes(int64_t n);
int dfx_inner_product(const double* d_a, const double* d_b, int64_t n,
                      void* d_work, size_t work_bytes, double* result,
                      void* stream);

/* ------------------------------------------------------------------ CG */
typedef struct dfx_cg_info
{
  int32_t iterations;
  int32_t status;          /* DFX_OK, DFX_ERR_NOT_CONVERGED, DFX_ERR_BREAKDOWN */
  double rnorm0_sq;        /* |r0|^2 */
  double rnorm_sq;         /* |r_k|^2 */
  int64_t kernel_launches; /* kernels this solve launched (graph nodes included) */
} dfx_cg_info;

/* Workspace of dfx_cg_solve for n scalar unknowns. */
size_t dfx_cg_workspace_bytes(int64_t n);

/* Jacobi-preconditioned CG (the demo's CG, cpp/demo/poisson_matrix_free/
 * main.cpp:84-132, with z = D^{-1} r; d_dinv == NULL gives plain CG).
 * Stops when |r|^2 / |r0|^2 < rtol^2. d_x holds the initial guess. FP64
 * throughout. The iteration runs as a CUDA graph of `graph_iters`
 * iterations (0: default) with device-side convergence tests. */
int dfx_cg_solve(const dfx_csr* A, const double* d_b, double* d_x,
                 const double* d_dinv, double rtol, int32_t max_iters,
                 int32_t graph_iters, void* d_work, size_t work_bytes,
                 dfx_cg_info* info, void* stream);

/* dfx_cg_solve for callers that cannot allocate memory. No counterpart in
 * the reference. Some callers may not allocate at all once they are
 * running: a host that has handed all device memory to its own pool and
 * solves between that set-up and its later graph capture, a plugin whose
 * host application owns every allocation, a real-time loop that forbids
 * allocation after start-up. This entry point calls no cudaMalloc,
 * cudaMallocHost, cudaFree or graph instantiation: its scratch (state,
 * reduction buffers and the vectors r, p, y) is a fixed 13 MiB array in
 * the library's device image, present on every GPU that loads the library
 * until the process exits, and it reads the solver state into pageable
 * host memory every `check_every` iterations (0: 20). Every call therefore
 * synchronises its stream: no call may be made while its stream (or the
 * legacy default stream) is being captured. At most 524288 scalar
 * unknowns; larger systems are rejected with DFX_ERR_INVALID. The first
 * call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current and keeps it for the
 * process; a host that calls cudaDeviceReset must not call this entry
 * point again afterwards. All calls share the one array, so calls whose
 * work overlaps on the GPU (other streams or host threads) race; serialise
 * them. Same iteration, stopping test and results as dfx_cg_solve. */
int dfx_cg_solve_noalloc(const dfx_csr* A, const double* d_b, double* d_x,
                         const double* d_dinv, double rtol, int32_t max_iters,
                         int32_t check_every, dfx_cg_info* info, void* stream);

/* ------------------------------------------ exterior facets, functionals */

/* Exterior facets of a tetrahedral mesh as (cell, local facet) pairs: the
 * integration domain of an exterior-facet integral on one rank
 * (mesh::exterior_facet_indices, mesh/utils.cpp:61-89, facets with one
 * attached cell; fem::compute_integration_domains, fem/utils.h:155-162).
 * Local facet f is the triangle opposite vertex f. facets: capacity
 * 8*num_cells int32; pairs sorted by (cell, facet); *num_facets = count.
 * Host function. */
int dfx_exterior_facets_tet(int32_t num_cells, const int32_t* cells, int32_t* facets,
                            int32_t* num_facets);

/* Interior facets of a tetrahedral mesh: the integration domain of an
 * interior-facet integral on one rank (fem::compute_integration_domains,
 * fem/utils.cpp:223-254: facets with two attached cells, each written as
 * (cell0, local facet0, cell1, local facet1)). A facet shared by more
 * than two cells is left out, as in the reference. facets: capacity
 * 8*num_cells int32; (cell0, facet0) < (cell1, facet1) within each
 * entry, entries sorted by (cell0, facet0); *num_facets = count. This
 * order is the library's own (the meshes here number no facets; the
 * reference lists facets by facet index): the same set and pairing, so
 * sums over the domain agree up to summation order. num_cells < 2^30.
 * Host function. */
int dfx_interior_facets_tet(int32_t num_cells, const int32_t* cells, int32_t* facets,
                            int32_t* num_facets);

/* Exterior-facet vector loop (fem/assemble_vector_impl.h:160-215,
 * 571-600): b += \int_F g v ds over the facets, L a DFX_FORM_SOURCE form
 * (g = its P1 coefficient f, or f_const[0]), scalar P1/P2. FP64 atomics. */
int dfx_assemble_vector_facets(const dfx_form* L, const int32_t* d_facets,
                               int32_t num_facets, double* d_b, void* stream);

/* Exterior-facet matrix loop (fem/assemble_matrix_impl.h:265-379):
 * A += \int_F alpha u v ds, a a DFX_FORM_FACET_MASS form, scalar P1/P2;
 * constrained rows and columns (d_bc) are skipped as in the cell loop.
 * d_map: the cell -> slot map of the cell integral (or NULL: row search). */
int dfx_assemble_matrix_facets(const dfx_form* a, const int32_t* d_facets,
                               int32_t num_facets, const dfx_csr* A,
                               const uint8_t* d_map, const int8_t* d_bc, void* stream);

/* Interior-facet vector loop (fem/assemble_vector_impl.h:252-360, the
 * interior_facet branch of assemble_vector): b += \int_F avg(g) avg(v) dS
 * over (cell0, facet0, cell1, facet1) quads (dfx_interior_facets_tet), L a
 * DFX_FORM_SOURCE form (g its P1 coefficient, or f_const[0]); each side
 * adds half. Scalar P1/P2, FP64 atomics; d_facets 16-byte aligned. */
int dfx_assemble_vector_interior_facets(const dfx_form* L, const int32_t* d_facets,
                                        int32_t num_facets, double* d_b, void* stream);

/* Interior-facet matrix loop (fem/assemble_matrix_impl.h:443-667): A +=
 * the macro-element tensor (cell0 dofs, then cell1 dofs) of a
 * DFX_FORM_FACET_JUMP form; constrained rows and columns (d_bc, may be
 * NULL) skipped as in the cell loop; insertion by binary search, so A's
 * pattern must hold the facet couplings (sparsitybuild::interior_facets:
 * build it from the macro elements). "Entry not in sparsity" otherwise. */
int dfx_assemble_matrix_interior_facets(const dfx_form* a, const int32_t* d_facets,
                                        int32_t num_facets, const dfx_csr* A,
                                        const int8_t* d_bc, void* stream);

/* Lifting of a facet integral (lift_bc, fem/assemble_vector_impl.h:363-414,
 * over a facet domain): b -= alpha A_F (g - x0) on the constrained columns
 * of each facet's element tensor. interior = 0: exterior (cell, facet)
 * pairs and a DFX_FORM_FACET_MASS form; interior = 1: quads and a
 * DFX_FORM_FACET_JUMP form. d_x0 may be NULL. */
int dfx_apply_lifting_facets(const dfx_form* a, const int32_t* d_facets, int32_t num_facets,
                             int32_t interior, double* d_b, const int8_t* d_bc,
                             const double* d_g, const double* d_x0, double alpha,
                             void* stream);

/* fem::assemble_scalar over cells (fem/assembler.h:173-215;
 * fem/assemble_scalar_impl.h:32-61) for the functionals M = a(u, u) of a
 * DFX_FORM_POISSON form (kappa |grad u|^2 + k2 u^2) and M = L(u) of a
 * DFX_FORM_SOURCE form (f u). u: FE function on the form's dofmap. The
 * sum is deterministic (fixed block and warp order). *value on the host;
 * synchronises `stream`. */
size_t dfx_assemble_scalar_workspace_bytes(int32_t num_cells);
int dfx_assemble_scalar(const dfx_form* M, const double* d_u, double* value,
                        void* d_work, size_t work_bytes, void* stream);

/* -------------------------------------------------------------- autotuner
 * No reference counterpart: the launch shapes of the assembly and CSR SpMV
 * kernels on this GPU. The library keeps one process-wide table of choices
 * per device and workload; a workload without an entry uses the defaults
 * (32 cells per block, 4 for elasticity; lanes per row from the mean row
 * length). */

/* Times the matrix assembly kernel with 16, 32 and 64 cells per block (2, 4
 * and 8 for elasticity), accumulating into d_scratch_vals (A->nnz*bs*bs
 * doubles; A's values are not touched). Records the fastest for this form
 * (kind, degree, mass term, number of cells) and mode, and returns it in
 * *best. ms (3 floats, may be NULL) receives each candidate's mean time per
 * assembly. Synchronises `stream`. */
int dfx_tune_assembly(const dfx_form* a, const dfx_csr* A, const uint8_t* d_map,
                      const int8_t* d_bc, int32_t mode, const int32_t* d_order,
                      const int32_t* colour_offsets, int32_t num_colours,
                      double* d_scratch_vals, int32_t* best, float* ms, void* stream);
/* Pin (cpb = one of the candidates) or reset (cpb = 0) the choice; read the
 * choice in force. */
int dfx_set_cells_per_block(const dfx_form* a, int32_t mode, int32_t cpb);
int dfx_get_cells_per_block(const dfx_form* a, int32_t mode, int32_t* cpb);

/* Row split of the scalar CSR SpMV (dfx_spmv and the CSR CG): times 4, 8,
 * 16 and 32 lanes per row on d_y = A d_x (d_y is overwritten), records the
 * fastest for matrices of this shape (rows, entries, dtype) and returns it
 * in *best_lanes. ms (4 floats, may be NULL) receives the mean times.
 * Synchronises `stream`. */
int dfx_tune_spmv(const dfx_csr* A, const void* d_x, void* d_y, int32_t* best_lanes,
                  float* ms, void* stream);
int dfx_set_spmv_lanes(const dfx_csr* A, int32_t lanes); /* 0: default */
int dfx_get_spmv_lanes(const dfx_csr* A, int32_t* lanes);
/* Forget every recorded choice. */
int dfx_tune_clear(void);
/* The recorded choices as rows of 6 int64, (device, what, k0, k1, k2,
 * value), in key order: what 1 = cells per block (k0 cells, k1 = 16 kind +
 * 4 degree + 2 mass + mode, k2 0), what 2 = lanes per row (k0 rows, k1
 * entries, k2 = 4 bs + dtype). With rows NULL only *num is written; with
 * fewer than *num rows of room, DFX_ERR_NO_MEMORY and *num = the count
 * needed. This is what a tuning cache file stores. */
int dfx_tune_export(int64_t* rows, int64_t cap, int64_t* num);
/* Add exported rows to the table, replacing entries of the same key. All
 * rows are checked first (device >= 0; what 1 with a value among its form
 * kind's candidates, what 2 with 4, 8, 16 or 32); on a bad row nothing is
 * added and DFX_ERR_INVALID names it. */
int dfx_tune_import(const int64_t* rows, int64_t num);

/* ---------------------------------------------------------------- timings
 * Named wall-clock timings of host work, accumulated per task for the life
 * of the process: common::Timer / TimeLogger (common/Timer.h:38-141,
 * common/TimeLogger.cpp:27-40). The host set-up above registers under the
 * reference's task names: "Build BoxMesh (tetrahedra)"
 * (mesh/generation.h:386), "Compute local part of mesh dual graph"
 * (mesh/graphbuild.cpp:575), "Reverse Cuthill-McKee ordering"
 * (graph/ordering.cpp:70), "Dofmap builder: build dofmap data"
 * (fem/dofmapbuilder.cpp:666), "Dofmap builder: compute dof reordering map"
 * (fem/dofmapbuilder.cpp:428) and "Build sparsity" (fem/utils.h:251; one
 * repetition per dfx_sparsity_create call, so the count pass and the fill
 * pass of one pattern are two). Device work is asynchronous and is timed
 * with CUDA events by its caller instead. */

/* One more repetition of `seconds` for `task` (a NUL-terminated name). */
int dfx_timing_record(const char* task, double seconds);
/* (repetitions, total seconds) of a task: dolfinx::timing
 * (common/timing.h:36-38). DFX_ERR_INVALID, "No timings registered for task
 * "<task>".", when it has none. */
int dfx_timing(const char* task, int32_t* count, double* total_seconds);
/* The tasks in byte-wise name order (dolfinx::timings(), common/timing.h:
 * 42-46): their number, and the i-th. name receives at most name_cap bytes
 * including the NUL (truncated if longer); *name_len the full length. */
int dfx_timing_num_tasks(int32_t* num);
int dfx_timing_task(int32_t i, char* name, int32_t name_cap, int32_t* name_len,
                    int32_t* count, double* total_seconds);
/* Forget every timing. */
int dfx_timing_clear(void);

/* ------------------------------------------------- sliced-ELL operator
 * The solver-side copy of a scalar MatrixCSR: rows sorted by length
 * within windows of `sigma` rows (a multiple of 32), the system renumbered
 * symmetrically with that permutation, 32-row slices stored column-major
 * so that every lane of a warp owns one row. No reference counterpart: it
 * is the GB300 layout behind MatrixCSR::mult inside the solvers
 * (la/MatrixCSR.h:877-946). FP32 operators may store columns as a first
 * column per row plus 16-bit deltas (DFX_ERR_UNSUPPORTED if a row has a
 * gap above 65535). A bs 3 matrix gives a 3x3-block operator (FP64 or
 * DFX_F32X2 values, 32-bit block columns, host build): slices of 32 block
 * rows, sigma counted in block rows, vectors of 3 nrows scalar entries.
 * The library owns the operator's device memory. */
typedef struct dfx_operator_s* dfx_operator;

int dfx_operator_create(const dfx_csr* A, int32_t sigma, int32_t value_dtype,
                        int32_t compress_cols, dfx_operator* op, void* stream);
/* Where dfx_operator_create_ex builds the structure. DFX_BUILD_AUTO (what
 * dfx_operator_create does): on the device, or on the host when a row has
 * more than 256 entries or sigma > 4096. DFX_BUILD_DEVICE refuses such
 * matrices with DFX_ERR_UNSUPPORTED. DFX_BUILD_HOST: the host builder.
 * Every place gives the same arrays bit for bit. */
enum
{
  DFX_BUILD_AUTO = 0,
  DFX_BUILD_DEVICE = 1,
  DFX_BUILD_HOST = 2
};
int dfx_operator_create_ex(const dfx_csr* A, int32_t sigma, int32_t value_dtype,
                           int32_t compress_cols, int32_t build, dfx_operator* op,
                           void* stream);
/* Refill the operator's values from A's FP64 values (after re-assembly). */
int dfx_operator_update_values(dfx_operator op, const dfx_csr* A, void* stream);
/* y = A x in the original numbering (x, y of the operator's dtype). */
int dfx_operator_apply(dfx_operator op, const void* d_x, void* d_y, void* stream);
/* y' = A' x' in the operator's own (renumbered) numbering: the bare SpMV
 * kernel the solvers run. */
int dfx_operator_apply_renumbered(dfx_operator op, const void* d_x, void* d_y, void* stream);
int dfx_operator_info(dfx_operator op, int64_t* nslots, int32_t* nslices,
                      const int32_t** d_perm);
int dfx_operator_destroy(dfx_operator op);
/* Free the values and scratch of an operator that owns its structure and
 * serves only as the source of shares (dfx_operator_share), e.g. a cached
 * structure whose requests each hold their own values. Afterwards the
 * operator can be shared, permuted, queried and destroyed; applying it,
 * refilling it or solving with it returns DFX_ERR_INVALID. */
int dfx_operator_release_values(dfx_operator op);
/* Device bytes the operator holds: its values and scratch, and for an
 * operator that owns its structure (not a share) the structure arrays. For
 * HBM accounting (no reference counterpart). */
int dfx_operator_device_bytes(dfx_operator op, size_t* bytes);
/* Launch shape of an FP32 operator's SpMV (no reference counterpart; an
 * autotuner knob): value pairs per load chunk of a lane, 2, 4 (default) or
 * 8. For a 3x3-block operator: 2, 4 or 8 (default) stand for 1, 2 or 4
 * block slots per round of a lane. Results are bitwise the same for every
 * choice. */
int dfx_operator_set_chunk(dfx_operator op, int32_t chunk);

/* Launch setting of the FP32 inner iteration (no reference counterpart),
 * for the calling host thread: on = 1 (default) runs each iteration as two
 * kernels, the SpMV and one cooperative kernel for the p.Ap reduction, the
 * x/r update with its dot products and the p update (grid-wide barriers in
 * place of kernel boundaries); on = 0 runs the four-kernel iteration. Same
 * recurrence; the dot products are summed in another fixed order. The
 * cooperative kernel holds every SM while it runs, so threads that solve
 * concurrently on several streams should switch it off. Applies to solves
 * the thread starts after the call. */
int dfx_set_cg_fused_update(int32_t on);
int dfx_get_cg_fused_update(int32_t* on);
/* Self-test of the fused update's grid barrier (no reference counterpart):
 * two cooperative blocks wait for a third arrival that never comes, so
 * their bounded waits run out (about a quarter of a second) and each
 * reports DFX_ERR_TIMEOUT instead of hanging. *gave_up = the number of
 * blocks that reported it (2 when the limit works). Synchronises the
 * device. */
int dfx_selftest_grid_barrier(int32_t* gave_up);

/* dfx_cg_solve on an FP64 operator (same iteration and stopping test). */
size_t dfx_cg_op_workspace_bytes(int64_t n);
int dfx_cg_solve_op(dfx_operator op, const double* d_b, double* d_x,
                    const double* d_dinv, double rtol, int32_t max_iters,
                    int32_t graph_iters, void* d_work, size_t work_bytes,
                    dfx_cg_info* info, void* stream);

/* Mixed-precision iterative refinement (no reference counterpart; it
 * wraps the demo's CG): r = b - A x, |r| and x += d in FP64 with op64;
 * corrections d come from Jacobi-PCG in FP32 (op32, FP32 vectors).
 *   DFX_IR_RESTART:  each correction is a fresh FP32 PCG solve of A d = r
 *                    to inner_rtol; max_outer caps the corrections.
 *   DFX_IR_RELIABLE: one FP32 PCG whose residual is replaced by the FP64
 *                    residual b - A x whenever it has dropped by inner_rtol
 *                    (reliable updates); x += d in FP64 at each replacement,
 *                    the search direction is kept; max_outer caps the
 *                    replacements, max_inner the FP32 iterations.
 *   DFX_IR_FLEXIBLE: FP64 flexible CG (one stored direction) whose
 *                    preconditioner is an FP32 PCG solve of A d = r to
 *                    inner_rtol (at most max_inner iterations each); the
 *                    outer vectors, products and update stay FP64. It
 *                    converges where the FP32 recurrence alone stalls
 *                    (FP32 rounding comparable to the smallest eigenvalue);
 *                    max_outer caps the outer iterations.
 * Stops when |b - A x|^2 / |b - A x0|^2 < rtol^2 evaluated in FP64 -- the
 * stopping test of dfx_cg_solve. op64 and op32 must be built from the same
 * matrix with the same sigma. */
enum dfx_ir_variant
{
  DFX_IR_RESTART = 0,
  DFX_IR_RELIABLE = 1,
  DFX_IR_FLEXIBLE = 2
};
typedef struct dfx_ir_info
{
  int32_t outer_iterations;
  int32_t inner_iterations;   /* total FP32 PCG iterations */
  int32_t status;
  int32_t reserved;
  double rnorm0_sq;
  double rnorm_sq;
  int64_t kernel_launches;    /* kernels this solve launched (graph nodes included) */
} dfx_ir_info;

size_t dfx_ir_workspace_bytes(int64_t n);
int dfx_ir_solve(dfx_operator op64, dfx_operator op32, const double* d_b, double* d_x,
                 const double* d_dinv, double rtol, double inner_rtol,
                 int32_t max_outer, int32_t max_inner, int32_t graph_iters,
                 int32_t variant, void* d_work, size_t work_bytes, dfx_ir_info* info,
                 void* stream);

/* dfx_operator whose structure (permutation, slices, columns, slot map) is
 * src's and whose values are its own: one structure per mesh, one set of
 * values per request. src must outlive its shares. */
int dfx_operator_share(dfx_operator src, dfx_operator* out);
/* dfx_operator_share with the values and scratch taken, in the order of
 * `stream`, from a stream-ordered pool the library keeps per device (no
 * reference counterpart). For servers that make and drop a share per
 * request: cudaMalloc and cudaFree would wait for the whole device each
 * time. Drop such a share with dfx_operator_destroy_async on a stream
 * ordered after every use of it (dfx_operator_destroy works too, but waits
 * for the device). Freed memory stays in the pool for the next shares until
 * dfx_operator_pool_trim. */
int dfx_operator_share_async(dfx_operator src, void* stream, dfx_operator* out);
int dfx_operator_destroy_async(dfx_operator op, void* stream);
/* Return the pool's unused memory to the device (waits for the device). */
int dfx_operator_pool_trim(void);
/* to_operator != 0: out[i] = in[perm[i]] (into the operator's numbering);
 * otherwise out[perm[i]] = in[i] (back to the original numbering). */
int dfx_operator_permute(dfx_operator op, const double* d_in, double* d_out,
                         int32_t to_operator, void* stream);

/* --------------------------------------------------------- batched CG
 * Serving path (no reference counterpart; it runs the demo's CG,
 * cpp/demo/poisson_matrix_free/main.cpp:84-132, for many systems at once).
 * One persistent launch advances every active system by up to `iterations`
 * PCG iterations, one CTA of 1024 threads per system, block reductions only;
 * the host retires finished systems and admits new ones between steps
 * (continuous batching). Vectors are in the operators' numbering
 * (dfx_operator_permute). mode 0: FP64 PCG on op64; mode 1: FP32 PCG on
 * op32 with FP64 reliable updates on op64 every time |r| drops by `delta`
 * (<= 0: 0.01). Stopping test |b - A x|^2 / |b - A x0|^2 < rtol^2, evaluated
 * in FP64. A system's result does not depend on the other systems. */
typedef struct dfx_batch_s* dfx_batch;
typedef struct dfx_batch_system
{
  dfx_operator op32;   /* FP32 operator (mode 1), or NULL */
  dfx_operator op64;   /* FP64 operator */
  const double* b;     /* right-hand side, operator numbering */
  double* x;           /* initial guess in, solution out, operator numbering */
  const double* dinv;  /* Jacobi inverse diagonal (operator numbering) or NULL */
  void* work;          /* dfx_batch_workspace_bytes(n, mode) bytes, 256-aligned */
  double rtol;
  double delta;
  int32_t max_iters;
  int32_t mode;
} dfx_batch_system;

size_t dfx_batch_workspace_bytes(int64_t n, int32_t mode);
int dfx_batch_create(int32_t capacity, dfx_batch* out);
int dfx_batch_destroy(dfx_batch b);
/* Put a system in a slot (its state restarts). */
int dfx_batch_set(dfx_batch b, int32_t slot, const dfx_batch_system* sys, void* stream);
int dfx_batch_clear(dfx_batch b, int32_t slot);
/* One launch over the set, unfinished slots; returns when it is done. */
int dfx_batch_step(dfx_batch b, int32_t iterations, int32_t* num_active, void* stream);
int dfx_batch_info(dfx_batch b, int32_t slot, dfx_cg_info* info, int32_t* done,
                   int32_t* replacements);

/* ------------------------------------------------ matrix-free Q4 action
 * The operator of the matrix-free Poisson demo (cpp/demo/poisson_matrix_free/
 * main.cpp:201-222; its form M = action(a, u), poisson.py:33-46) for
 * a(u,v) = \int kappa grad u . grad v on Lagrange Q4 hexahedra, applied by
 * sum factorisation: a structured nx x ny x nz hexahedral mesh with
 * trilinear geometry (vertices lexicographic, x fastest), Gauss-Lobatto-
 * Legendre nodes, Gauss-Legendre 5^3 quadrature, nodes lexicographic on the
 * (4nx+1)(4ny+1)(4nz+1) lattice. y = A u on interior nodes (boundary
 * entries of u read as 0), y = u on boundary nodes: homogeneous Dirichlet
 * rows set to the identity. */
typedef struct dfx_q4_mesh
{
  int32_t nx, ny, nz;
  const double* verts;  /* ((nx+1)(ny+1)(nz+1), 3) vertex coordinates */
  double kappa;
  /* Optional (NULL: formed on the fly): the cells' edge vectors in FP32,
   * 36 floats per cell, 16-byte aligned, written by dfx_q4_edges. Used by
   * the FP32 action only; results are bitwise the same either way. */
  const float* edges32;
  /* Optional (NULL: formed on the fly): the geometric factor of every
   * quadrature point, G = w kappa adj(J) adj(J)^T / |det J| (symmetric, 6
   * values: 00, 01, 02, 11, 12, 22), written by dfx_q4_geometry. 750
   * values per cell, [cell][6][125], point x + 5 y + 25 z, cells
   * lexicographic. geom32 serves the FP32 action, geom64 the FP64 one; they
   * agree with the on-the-fly path to the precision's rounding. No
   * counterpart in the reference, which forms the geometry in every cell
   * kernel call: a cache of 3 KB (FP32) or 6 KB (FP64) per cell. */
  const float* geom32;
  const double* geom64;
} dfx_q4_mesh;

int64_t dfx_q4_num_dofs(const dfx_q4_mesh* mesh);
/* Writes the 36 * nx * ny * nz FP32 edge components of dfx_q4_mesh.edges32
 * (no counterpart in the reference: a cache of per-cell geometry). */
int dfx_q4_edges(const dfx_q4_mesh* mesh, float* d_edges, void* stream);
/* Writes the 750 * nx * ny * nz geometric factors of dfx_q4_mesh.geom32
 * (dtype DFX_F32) or .geom64 (DFX_F64), computed in that precision from the
 * edge vectors rounded once from the FP64 vertices. */
int dfx_q4_geometry(const dfx_q4_mesh* mesh, int32_t dtype, void* d_geom, void* stream);
/* y = A u; u, y of `dtype` (DFX_F64 or DFX_F32; FP32 forms the geometry
 * and contractions in FP32 from FP64 vertex differences). */
int dfx_q4_action(const dfx_q4_mesh* mesh, int32_t dtype, const void* d_u, void* d_y,
                  void* stream);
/* y = A u in FP32 with every 1D basis contraction on the tensor cores
 * (tcgen05.mma kind::tf32; each operand split as hi + lo so that the
 * three products hi*hi + lo*hi + hi*lo keep FP32-level accuracy); the
 * geometry stays on the CUDA cores. Same operator and results (to FP32
 * rounding) as dfx_q4_action(DFX_F32). */
int dfx_q4_action_tc(const dfx_q4_mesh* mesh, const float* d_u, float* d_y, void* stream);
/* Synchronises `stream`; DFX_ERR_TIMEOUT if a tensor-core kernel stopped
 * early because an MMA completion wait ran out (its y is then invalid). */
int dfx_q4_tc_check(void* stream);
/* CG on the Q4 action (the demo's unpreconditioned CG, main.cpp:84-132).
 * mode 0: FP64 throughout; mode 1: FP32 action and vectors with FP64
 * reliable updates (FP64 action for the residual, x += d in FP64) when |r|
 * has dropped by `delta`; mode 2: mode 1 with the tensor-core FP32 action
 * (dfx_q4_action_tc). Stops at |b - A x|^2/|b - A x0|^2 < rtol^2 in FP64. */
size_t dfx_q4_cg_workspace_bytes(int64_t n, int32_t mode);
int dfx_q4_cg_solve(const dfx_q4_mesh* mesh, const double* d_b, double* d_x, double rtol,
                    int32_t max_iters, int32_t mode, double delta, int32_t graph_iters,
                    void* d_work, size_t work_bytes, dfx_cg_info* info, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DFX_GPU_H */
