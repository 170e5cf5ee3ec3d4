/* fluidity_gb300.h -- C-ABI of the GB300 (sm_103a) CG assembly + Krylov path.
 *
 * Drop-in boundary for Fluidity's continuous-Galerkin scalar hot path:
 * the element loop of assemble/Advection_Diffusion_CG.F90 (and the P1/P2
 * pressure Laplacians built by the same kernels), the csr_matrix sparsity and
 * colouring it uses, strong Dirichlet conditions, and the petsc_solve Krylov
 * solve on the assembled system.  A Fortran caller binds these entry points
 * with ISO_C_BINDING (fluidity_gb300/fortran/fl_gpu_bindings.F90) and passes
 * c_loc() pointers to the arrays it already owns:
 *
 *   csr_sparsity  findrm(N+1), colm(nnz), centrm(N)  1-based int32
 *                 (femtools/Sparse_Tools.F90:48-111)
 *   csr_matrix    val(nnz) real64, inactive%ptr(N) logical
 *   scalar_field  val(N) real64
 *   vector_field  val(3,N) real64, xyz interleaved per node
 *   mesh_type     ndglno(loc*E) int32, element-major
 *                 (femtools/Fields_Data_Types.F90:61-76,187-216)
 *
 * Conventions: plain pointers and sizes; no CUDA or torch types in the
 * signatures (streams are passed as void*).  Functions named fl_gpu_* take
 * HOST pointers and copy in/out; functions named fl_dev_* take DEVICE pointers
 * and run on the given stream (NULL = the mesh handle's stream; the legacy
 * default stream is passed as cudaStreamLegacy).  Every
 * function returns an fl_status; fl_last_error() describes the last failure
 * of the calling thread.  Indices follow `index_base` (1 = Fortran, 0 = C).
 * The calls on one handle share its scratch buffers (element records, staging
 * arrays): issue them on one stream, or order them across streams.
 */
#ifndef FLUIDITY_GB300_H
#define FLUIDITY_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Usage errors (>0) correspond to FLAbort/FLExit in the
 * reference (include/fdebug.h:56-57); FL_ERR_OUTSIDE_PATTERN is csr_addto's
 * "Attempting to set value in matrix outside sparsity pattern."
 * (femtools/Sparse_Tools.F90:2646).  Solver divergence is not an error: it is
 * reported as a negative KSPConvergedReason in fl_solve_report::reason. */
enum fl_status {
  FL_OK = 0,
  FL_ERR_ARG = 1,
  FL_ERR_CUDA = 2,
  FL_ERR_OUTSIDE_PATTERN = 3,
  FL_ERR_TIMEOUT = 4,
  FL_ERR_COLOURS = 5,
  FL_ERR_NOMEM = 6,
  FL_ERR_UNSUPPORTED = 7
};

/* KSPConvergedReason values used by the device solvers (PETSc, the third-party
 * library called at femtools/Solvers.F90:1251; checked by ConvergenceCheck,
 * femtools/Solvers.F90:1369-1479). */
enum fl_reason {
  FL_CONVERGED_RTOL = 2,
  FL_CONVERGED_ATOL = 3,
  FL_DIVERGED_NULL = -2,
  FL_DIVERGED_ITS = -3,
  FL_DIVERGED_DTOL = -4,
  FL_DIVERGED_BREAKDOWN = -5,
  FL_DIVERGED_INDEFINITE_PC = -8,
  FL_DIVERGED_NANORINF = -9,
  FL_DIVERGED_INDEFINITE_MAT = -10
};

/* Message describing the last non-OK status returned on this thread. */
const char* fl_last_error(void);

/* ---------------------------------------------------------------- meshes -- */

typedef struct fl_mesh_t* fl_mesh;

typedef struct {
  int32_t nodes;            /* node_count of the field mesh (matrix rows)   */
  int32_t elements;         /* element_count                                */
  int32_t loc;              /* nodes per element: 4 (P1) or 10 (P2)         */
  int32_t index_base;       /* 1: Fortran ndglno; 0: C                      */
  const int32_t* ndglno;    /* loc*elements field-mesh connectivity         */
  int32_t x_nodes;          /* node_count of the coordinate (P1) mesh       */
  const int32_t* x_ndglno;  /* 4*elements coordinate/topology connectivity  */
  const double* coords;     /* 3*x_nodes, positions%val(3,N)                */
} fl_mesh_desc;

/* Registers a mesh: uploads connectivity and coordinates, builds on the GPU the
 * first-order sparsity (replaces get_csr_sparsity_firstorder ->
 * make_sparsity, femtools/Sparsity_Patterns_Meshes.F90:76,
 * femtools/Sparsity_Patterns.F90:47) and the COLOURING_CG1 element colouring
 * (replaces get_mesh_colouring, femtools/Colouring.F90:85), both bit-exact with
 * the reference, and caches them on the handle as the reference caches them
 * in state / on the topology mesh. */
int fl_gpu_mesh_register(const fl_mesh_desc* desc, fl_mesh* out);
int fl_gpu_mesh_destroy(fl_mesh mesh);

/* A handle holding only a square CSR pattern (n rows, findrm(n+1), colm, each
 * row's columns strictly ascending; index_base as elsewhere) and no elements:
 * for solving a system read from a file (the matrixdump that
 * DumpMatrixEquation writes, femtools/Petsc_Tools.F90:1487-1504, and that
 * tools/petsc_readnsolve.F90 reads) with fl_gpu/dev_petsc_solve and
 * fl_dev_csr_mult.  Assembly on such a handle returns FL_ERR_ARG. */
int fl_gpu_pattern_register(int32_t n, const int32_t* findrm, const int32_t* colm, int32_t index_base,
                            fl_mesh* out);
/* Sizes of the cached structures: entries of the sparsity and colour count. */
int fl_gpu_mesh_info(fl_mesh mesh, int64_t* nnz, int32_t* ncolours);

/* Copies the cached csr_sparsity out (findrm(N+1), colm(nnz), centrm(N)) in
 * the requested index base.  centrm of a row without diagonal is 0 in base 1
 * (lists2csr_sparsity, femtools/Sparsity_Patterns.F90:414-426) and -1 in base 0. */
int fl_gpu_sparsity_copy(fl_mesh mesh, int32_t* findrm, int32_t* colm, int32_t* centrm,
                         int32_t index_base);

/* Copies the colouring out: colour(E) 1-based colours per element, and the
 * colour sets as colour_ptr(ncolours+1) offsets into colour_elems(E), elements
 * ascending within a set (colour_sets, femtools/Colouring.F90:250-262). */
int fl_gpu_colouring_copy(fl_mesh mesh, int32_t* colour, int32_t* colour_ptr,
                          int32_t* colour_elems, int32_t index_base);

/* Node numbering of the P2 mesh derived from a P1 tet connectivity (replaces
 * make_global_numbering, femtools/Global_Numbering.F90:291-634, serial case),
 * computed on the GPU and bit-exact: vertices in first-touch element order,
 * then edges in (old node, neighbour ascending) order.  ndglno_p2 has
 * 10*elements entries in number_tets_lagrange local order
 * (femtools/Element_Numbering.F90:389-472); *n2 receives the node count. */
int fl_gpu_make_global_numbering_p2(int32_t nvert, int32_t elements, const int32_t* ndglno_p1,
                                    int32_t index_base, int32_t* ndglno_p2, int32_t* n2);

/* ------------------------------------------------------------- assembly -- */

/* Options of assemble_advection_diffusion_cg read from the options tree
 * (assemble/Advection_Diffusion_CG.F90:384-465). */
typedef struct {
  double theta;              /* temporal_discretisation/theta               */
  double dt;                 /* timestep                                    */
  double beta;               /* conservative_advection                      */
  int32_t have_mass;         /* .not. exclude_mass_terms                    */
  int32_t lump_mass;         /* lump_mass_matrix                            */
  int32_t have_advection;    /* .not. exclude_advection_terms               */
  int32_t have_diffusivity;
  int32_t isotropic_diffusivity;
  int32_t have_source;
  int32_t have_absorption;
  int32_t quad_degree;       /* quadrature degree of the mesh (2 or 4)      */
  double diffusivity[9];     /* constant diffusivity tensor, (i,j) row-major */
  int32_t integrate_advection_by_parts;  /* spatial_discretisation/
                                continuous_galerkin/advection_terms/
                                integrate_advection_by_parts: element term
                                -(grad N_i . u) N_j - (1 - beta) N_i N_j div u
                                (:1019-1057) instead of N_i u . grad N_j
                                + beta N_i N_j div u, plus the surface term of
                                fl_dev_assemble_advdif_faces                 */
  int32_t pad;
} fl_advdif_params;

/* Nodal fields.  t, source, absorption live on the field mesh; velocity lives
 * on the coordinate mesh (3 values per node).  NULL = absent (t = 0). */
typedef struct {
  const double* t;
  const double* velocity;
  const double* source;
  const double* absorption;
} fl_fields;

/* Element loop of assemble_advection_diffusion_cg
 * (assemble/Advection_Diffusion_CG.F90:560-598 -> element kernel :702-865 ->
 * addto, femtools/Sparse_Tools.F90:2680): zeroes val/rhs, then adds every
 * element's matrix and right-hand side into the csr_matrix values (pattern of
 * the handle) colour by colour, elements ascending within a colour, so the
 * sums are deterministic.  Host pointers: val(nnz), rhs(N).  With page-locked
 * val and rhs, the P1 diffusion forms (diagonal diffusivity) on meshes of at
 * least about 1 M matrix entries run in row chunks of about 4 MB of val:
 * field uploads, assembly and the copies of finished chunks back overlap,
 * and the results are the bits of the device entry point. */
int fl_gpu_assemble_advdif_cg(fl_mesh mesh, const fl_advdif_params* params,
                              const fl_fields* fields, double* val, double* rhs);
/* Device-pointer form of the same call (all field pointers device). */
int fl_dev_assemble_advdif_cg(fl_mesh mesh, const fl_advdif_params* params,
                              const fl_fields* fields, double* val, double* rhs,
                              void* stream);

/* Surface elements of the field mesh with their boundary conditions: the
 * input of the surface loop of assemble_advection_diffusion_cg
 * (assemble/Advection_Diffusion_CG.F90:608-640; get_entire_boundary_condition
 * with the types neumann, weakdirichlet, internal, robin).  Face nodes are in
 * the triangle's local order: P1 (floc 3) the three vertices; P2 (floc 6)
 * vertex 1, edge 12, vertex 2, edge 13, edge 23, vertex 3 (the triangle
 * numbering of femtools/Element_Numbering.F90).  xfaces holds the three
 * vertices on the coordinate mesh in the same vertex order.  All pointers are
 * device pointers for fl_dev_* and host pointers for fl_gpu_*. */
typedef struct {
  int32_t nfaces;
  int32_t floc;              /* nodes per face: 3 (P1 field) or 6 (P2)      */
  int32_t index_base;        /* 0 or 1 for faces, xfaces and face_ele       */
  int32_t pad;
  const int32_t* faces;      /* nfaces x floc field nodes (face_global_nodes) */
  const int32_t* xfaces;     /* nfaces x 3 coordinate vertices              */
  const int32_t* face_ele;   /* nfaces: the element of each face (face_ele);
                                needed with advection by parts (normals)    */
  const int32_t* bc_type;    /* nfaces: 0 none, 1 neumann, 2 weakdirichlet,
                                3 internal (skipped), 4 robin               */
  const double* bc_value;    /* nfaces x floc: t_bc at the face nodes
                                (neumann flux, robin value, weak Dirichlet
                                value); may be NULL when no face needs it   */
  const double* bc_value2;   /* nfaces x floc: t_bc_2 (robin coefficient)   */
} fl_face_bcs;

/* The surface loop of assemble_advection_diffusion_cg, added into an
 * assembled system (after fl_*_assemble_advdif_cg, before the strong
 * Dirichlet conditions, the reference's order): for every face in order,
 * unless internal, assemble_advection_diffusion_face_cg
 * (Advection_Diffusion_CG.F90:1228-1286) with add_advection_face_cg
 * (:1288-1342; when advection is integrated by parts: the face matrix
 * int N_i N_j (u.n) enters the matrix with dt*theta, or for weak Dirichlet
 * faces the rhs with theta*(g - t); the rhs loses its product with t) and
 * add_diffusivity_face_cg (:1344-1378; neumann: rhs += int N_i g; robin: the
 * same plus int N_i N_j g2 in the matrix with dt*theta and its product with
 * t subtracted from the rhs).  Nothing happens unless advection is by parts
 * or a diffusivity is present (:608-611).  A weak Dirichlet face with a
 * diffusivity is the reference's FLExit: FL_ERR_ARG (the system is then
 * partly updated).  The sums are deterministic: each row adds its faces in
 * ascending order.  Face quadrature: the triangle rule of params->quad_degree
 * (Quadrature.F90 construct_tri_quadratures).  Device pointers: fields->t and
 * fields->velocity (P1, on the coordinate mesh) as in the element loop. */
int fl_dev_assemble_advdif_faces(fl_mesh mesh, const fl_advdif_params* params, const fl_face_bcs* faces,
                                 const fl_fields* fields, double* val, double* rhs, void* stream);
/* Host-pointer form (val and rhs are read and updated in place). */
int fl_gpu_assemble_advdif_faces(fl_mesh mesh, const fl_advdif_params* params, const fl_face_bcs* faces,
                                 const fl_fields* fields, double* val, double* rhs);

/* Failure injection for tests of the bounded device waits (no counterpart in
 * the reference, whose loops do not wait on other threads).  Three kernels
 * wait on flags other threads set: the colouring dataflow of
 * fl_gpu_mesh_register (an element waits for the colours of its lower
 * neighbours; limit about 2 s), the fused P1 pass (row tile 3; a row item
 * waits for the element items it reads; limit 2^22 polls) and the
 * cooperative GMRES solve (schedule 2; its blocks meet at grid barriers;
 * limit 1 s per barrier).  After this call, in this process: wait_ms > 0
 * bounds each such wait to about wait_ms milliseconds, and withhold >= 0
 * keeps one flag unset -- the colour of element `withhold`, the completion of
 * element-item group `withhold`, or the barrier arrivals of block `withhold`
 * of the cooperative solve (which leaves at once) -- so that the waits on it
 * run out.  The waiting side then records FL_ERR_TIMEOUT and stops; every
 * kernel finishes, the call returns FL_ERR_TIMEOUT ("a bounded device wait ran
 * out"), the CUDA context and other handles stay usable, and the next call
 * without the hook gives the normal results.  fl_set_wait_test(-1, 0) switches
 * the hook off; a withheld flag needs wait_ms > 0. */
int fl_set_wait_test(int32_t withhold, double wait_ms);

/* Allocation-free form of fl_dev_assemble_advdif_cg for the P1 diffusion
 * (pressure-Poisson) case: diffusivity with optional source and consistent
 * mass, no advection or absorption, on a P1 field mesh.  No counterpart in the
 * reference.  It exists for callers that cannot allocate device memory when
 * they assemble -- an application whose memory manager has already reserved
 * the device, or a loop that must not call cudaMalloc because it can
 * synchronise the device.  The call allocates nothing: its element-matrix
 * scratch is a fixed array inside the library sized for at most 131072
 * elements (14.7 MB held on every GPU that loads the library); larger meshes
 * are rejected with FL_ERR_ARG.  The first call on a device also looks up
 * that array's device address and uploads the reference-element tables
 * (then waits for the device), so make the first call on each device before
 * any stream capture.  Every call waits for its stream before it returns (it
 * reads the pattern-error flag back).  Every call shares the array, so calls
 * whose GPU work overlaps (other streams or threads) race.  After
 * cudaDeviceReset the library must be unloaded and loaded again, like every
 * mesh handle.  Device pointers; the results agree with
 * fl_dev_assemble_advdif_cg's within rounding (that entry point computes the
 * isotropic and diagonal-diffusivity forms in double-float, this one in
 * FP64), and bitwise for a full diffusivity tensor. */
int fl_dev_assemble_p1_diffusion_noalloc(fl_mesh mesh, const fl_advdif_params* params,
                                         const fl_fields* fields, double* val, double* rhs,
                                         void* stream);

/* Strong Dirichlet (apply_dirichlet_conditions_scalar,
 * femtools/Boundary_Conditions.F90:1983-2025): marks rows inactive
 * (csr_set_inactive_rows, femtools/Sparse_Tools.F90:2136) and sets
 * rhs(b) = (g - t(b))/dt, or rhs(b) = g when dt <= 0.  inactive(N) is one
 * byte per row (0/1).  t may be NULL (zero). */
int fl_gpu_apply_dirichlet(fl_mesh mesh, int32_t nb, const int32_t* nodes, int32_t index_base,
                           const double* g, const double* t, double dt, double* rhs,
                           uint8_t* inactive);
int fl_dev_apply_dirichlet(fl_mesh mesh, int32_t nb, const int32_t* nodes, int32_t index_base,
                           const double* g, const double* t, double dt, double* rhs,
                           uint8_t* inactive, void* stream);

/* ---------------------------------------------------------------- solve -- */

/* Solver options read by petsc_solve_setup / setup_ksp_from_options
 * (femtools/Solvers.F90:1566-1660). */
typedef struct {
  int32_t ksp_type;          /* 0 = cg, 1 = gmres                           */
  int32_t restart;           /* gmres restart (schema default 30)           */
  double rtol;               /* relative_error                              */
  double atol;               /* absolute_error (default 0)                  */
  double dtol;               /* divergence tolerance (PETSc default 1e5)    */
  int32_t max_its;           /* max_iterations                              */
  int32_t start_from_zero;   /* start_from_zero                             */
  int32_t precision;         /* 0 = fp64; 1 = fp32 inner CG solves inside
                                fp64 iterative refinement (restarted);
                                2 = fp32 CG with reliable updates: fp64
                                refinement of the solution and residual
                                whenever the fp32 residual has dropped
                                tenfold, without restarting the fp32
                                Krylov space; the convergence test runs on
                                the fp64 residual (CG only)                  */
  double inner_rtol;         /* inner relative tolerance (precision = 1)    */
  int32_t norm_type;         /* KSPSetNormType: 0 = preconditioned ||B r||
                                (PETSc's default for CG and GMRES with left
                                Jacobi); 1 = unpreconditioned ||r||, CG only
                                (every precision), so rtol bounds the true
                                relative residual ||b - A x|| / ||b||        */
  int32_t schedule;          /* how an FP64 GMRES solve is launched:
                                0 = automatic (1 above FL_PERSIST_MAX_ROWS
                                rows, else 2); 1 = one kernel launch per
                                Arnoldi phase, each restart cycle replayed
                                as a CUDA graph; 2 = the whole solve in one
                                cooperative launch, the blocks meeting at
                                grid barriers (latency-bound small systems;
                                when the blocks' slices of the Krylov basis
                                do not fit in shared memory, 1 is used).
                                Other solves ignore it.                      */
} fl_solver_opts;

/* Largest system (rows) that schedule 0 solves in one cooperative launch. */
#define FL_PERSIST_MAX_ROWS 81920

typedef struct {
  int32_t iterations;        /* KSPGetIterationNumber (inner total if mixed) */
  int32_t reason;            /* KSPConvergedReason                          */
  double final_rnorm;        /* last preconditioned residual norm           */
  double rnorm0;             /* norm the relative tolerance scales          */
  double true_rel_residual;  /* ||b - A x|| / ||b|| recomputed in fp64      */
  int32_t outer_iterations;  /* refinement steps (precision = 1 or 2)       */
  int32_t pad;
} fl_solve_report;

/* petsc_solve on the handle's csr_matrix (femtools/Solvers.F90:111-187):
 * inactive rows become ghost rows (Petsc_Tools.F90:256-298) carrying the
 * diagonal ghost_pivot (Petsc_Tools.F90:960-985), ghost columns are lifted
 * into the rhs (Solvers.F90:1072-1104), CG or GMRES(restart) with Jacobi
 * preconditioning runs on the device with PETSc's default convergence test,
 * and ghost nodes take their rhs value afterwards (Petsc_Tools.F90:726-730).
 * Host pointers: val(nnz), inactive(N) or NULL, rhs(N), x(N) (initial guess
 * unless start_from_zero; solution on return). */
int fl_gpu_petsc_solve(fl_mesh mesh, const fl_solver_opts* opts, const double* val,
                       const uint8_t* inactive, const double* rhs, double* x,
                       fl_solve_report* report);
int fl_dev_petsc_solve(fl_mesh mesh, const fl_solver_opts* opts, const double* val,
                       const uint8_t* inactive, const double* rhs, double* x,
                       fl_solve_report* report, void* stream);

/* One step of solve_field_equation_cg on the device
 * (assemble/Advection_Diffusion_CG.F90:127-174): fl_dev_assemble_advdif_cg
 * into val/rhs, fl_dev_apply_dirichlet in rate-of-change form (inactive
 * cleared first; rhs = (g - t) / dt with fields->t and params->dt),
 * fl_dev_petsc_solve for delta from zero change, then t_new = t + dt delta
 * (t_new may be fields->t).  val(nnz), rhs(N), inactive(N) and delta(N) are
 * caller-owned device scratch.  The same kernels as the three calls, so the
 * same bits; a pattern miss or a boundary node out of range is reported once,
 * after the step, instead of after each stage. */
int fl_dev_solve_field_equation_cg(fl_mesh mesh, const fl_advdif_params* params, const fl_fields* fields,
                                   int32_t nb, const int32_t* bc_nodes, int32_t index_base,
                                   const double* bc_values, const fl_solver_opts* opts, double* val,
                                   double* rhs, uint8_t* inactive, double* delta, double* t_new,
                                   fl_solve_report* report, void* stream);

/* Initial guess for a solve in a sequence of solves (no counterpart in the
 * reference, which starts from the previous solution or from zero): the
 * projection method of P. F. Fischer (1998).  Given k (1..8) basis vectors
 * -- earlier solutions, a network's prediction -- x0 = V a where
 * (V^T A V) a = V^T b, with A and b the ghost-reduced system
 * fl_dev_petsc_solve solves (inactive rows and columns dropped, b = rhs
 * lifted by the inactive values), minimises the A-norm of x0's error over
 * span(V), the norm CG minimises; ghost rows of x0 take the rhs.  Basis
 * vectors in the span of earlier ones are dropped (LDL^T pivot below 1e-13
 * of its diagonal).  basis: a host array of k device pointers; coef (host,
 * k values, may be NULL) receives a.  Device pointers otherwise; the call
 * waits for its stream once (the k x k system is solved on the host). */
int fl_dev_projected_guess(fl_mesh mesh, const double* val, const uint8_t* inactive, const double* rhs,
                           int32_t k, const double* const* basis, double* x0, double* coef, void* stream);

/* y = A x on the handle's pattern (csr_mult, femtools/Sparse_Tools.F90:3822);
 * device pointers. */
int fl_dev_csr_mult(fl_mesh mesh, const double* val, const double* x, double* y, void* stream);

/* ------------------------------------------------------ tiles / batches -- */

/* Assembly tile autotuner (no counterpart in the reference, whose element
 * loop has no tiles).  Times the assembly of `params`/`fields` on the mesh
 * under each element-pass tile (128 or 256 threads per block x 4..32 blocks
 * per SM) and each row-pass tile (index 0..2: 64/128/256 rows per block for
 * P1, 32/64/128 for P2), keeps the fastest on the handle for later calls and
 * writes it to tiles[3] (may be NULL).  The tiles regroup independent work
 * only: val and rhs are identical under every choice and hold the assembled
 * system on return.  Device pointers, as fl_dev_assemble_advdif_cg. */
int fl_dev_autotune_assembly(fl_mesh mesh, const fl_advdif_params* params, const fl_fields* fields,
                             double* val, double* rhs, void* stream, int32_t* tiles);
int fl_set_assembly_tiles(fl_mesh mesh, int32_t elem_block, int32_t elem_blocks_per_sm, int32_t row_tile);
int fl_get_assembly_tiles(fl_mesh mesh, int32_t* tiles);

/* Batched steps (no single counterpart in the reference: they stand for many
 * solve_field_equation_cg calls, Advection_Diffusion_CG.F90:127-174, on
 * fields sharing one mesh or on several meshes).  A member is one step:
 * assembly as fl_dev_assemble_advdif_cg, strong Dirichlet conditions as
 * fl_dev_apply_dirichlet (inactive is cleared first), and an FP64 CG or
 * GMRES(restart) + Jacobi solve as fl_dev_petsc_solve into x.  All pointers
 * are DEVICE pointers owned by the caller and must stay valid while the batch
 * exists.  fl_batch_run executes every member as one branch of a CUDA graph
 * (assembly, conditions, set-up and the first iterations), then replays a
 * second graph of further iterations until every member has converged or
 * reached max_its, and fills reports[member] in the order of fl_batch_add.
 * The first run (and the first after an fl_batch_add) autotunes the tiles of
 * each mesh not tuned yet, builds the graphs and may allocate; later runs
 * re-execute the same graphs on the arrays' current contents.  Results are
 * identical to the unbatched entry points called member by member. */
typedef struct fl_batch_t* fl_batch;
int fl_batch_create(fl_batch* batch);
int fl_batch_add(fl_batch batch, fl_mesh mesh, const fl_advdif_params* params, const fl_fields* fields,
                 int32_t nb, const int32_t* bc_nodes, int32_t index_base, const double* bc_values,
                 const fl_solver_opts* opts, double* val, double* rhs, uint8_t* inactive, double* x);
int fl_batch_run(fl_batch batch, void* stream, fl_solve_report* reports);
int fl_batch_size(fl_batch batch);
int fl_batch_destroy(fl_batch batch);

/* ----------------------------------------------- AMG preconditioner -- */

/* Smoothed-aggregation algebraic multigrid for CG, the GPU counterpart of
 * the gamg preconditioner of petsc_solve's options (femtools/Solvers.F90:
 * 1827-1969, PETSc PCGAMG with its default structure):
 *   - aggregates from a distance-2 maximal independent set of the matrix graph;
 *   - one Jacobi smoothing of the piecewise-constant prolongator;
 *   - Galerkin coarse operators;
 *   - Chebyshev(2)-Jacobi smoothing;
 *   - a dense solve on the coarsest level (at most 512 rows).
 * fl_amg_create builds the hierarchy for the matrix val (device, on the
 * mesh's pattern) with the inactive (Dirichlet) rows of `inactive` (device,
 * may be NULL) treated as petsc_solve treats them.  Both arrays must stay
 * valid and unchanged while the handle is used; like cache_solver_context,
 * one hierarchy serves many right-hand sides.  fl_amg_solve runs CG on that
 * system with the hierarchy as preconditioner: ghost rows, rhs lifting and
 * PETSc's default convergence test on the preconditioned residual norm as
 * fl_dev_petsc_solve (opts: ksp_type 0, precision 0; report->outer_iterations
 * returns the number of levels).  Device pointers; the hierarchy and the
 * solve are deterministic. */
typedef struct fl_amg_t* fl_amg;
int fl_amg_create(fl_mesh mesh, const double* val, const uint8_t* inactive, void* stream, fl_amg* amg);
int fl_amg_solve(fl_amg amg, const fl_solver_opts* opts, const double* rhs, double* x,
                 fl_solve_report* report, void* stream);
int fl_amg_levels(fl_amg amg, int32_t* levels, int64_t* rows, int64_t* nnz, int32_t capacity);
/* Norm of the convergence test: 0 (default) the preconditioned residual
 * ||B r||, PETSc's default for CG; 1 the residual ||r|| itself
 * (KSP_NORM_UNPRECONDITIONED), so that rtol bounds ||b - A x|| / ||b||. */
int fl_amg_set_norm(fl_amg amg, int32_t unpreconditioned);
/* Arithmetic of the V-cycle: 0 (default) FP64; 1 FP32 operators and vectors
 * inside the cycle (a single-precision preconditioner for the FP64 CG, whose
 * residuals, dot products and convergence test stay in FP64). */
int fl_amg_set_precision(fl_amg amg, int32_t fp32);
int fl_amg_destroy(fl_amg amg);

/* ------------------------------------------------- learned warm start -- */

/* Message-passing network that predicts the next pressure of a sequence of
 * Poisson solves, used as the initial guess of fl_dev_petsc_solve (no
 * counterpart in the reference).  Node features: previous two pressures p1,
 * p2, the right-hand side b and the coordinates; three message-passing layers
 * of width 64 over the mesh's sparsity graph; BF16 weights and activations
 * with FP32 accumulation on the tensor cores; prediction
 * 2 p1 - p2 + max|p1| * output.  Parameters are one flat FP32 vector of
 * fl_gnn_num_params() entries:
 *   We[64][16] be[64] | 3 x (Wl[64][128] bl[64]) | wd[64] bd[1]
 * (Wl columns 0..63 act on the node's own state, 64..127 on the mean of its
 * neighbours').  All field pointers are DEVICE pointers of N doubles on a P1
 * mesh.  mask (N bytes, 1 = node counts in the loss; NULL = all) and nact
 * (its number of ones) select the nodes of the loss: the mean squared error
 * of the prediction normalised by max|p1|.  fl_gnn_gradients returns that
 * loss and its gradient (host arrays); fl_gnn_train_step applies one Adam
 * step (beta 0.9, 0.999) with learning rate lr and, if loss_dev is not NULL,
 * writes the step's sum of squared errors to that device float. */
typedef struct fl_gnn_t* fl_gnn;
int fl_gnn_num_params(void);
int fl_gnn_create(fl_mesh mesh, fl_gnn* net);
int fl_gnn_destroy(fl_gnn net);
int fl_gnn_set_weights(fl_gnn net, const float* weights, int32_t count);
/* Loss of the following gradient and training calls: val = NULL (default)
 * selects the mean squared error; a device pointer to the assembled matrix
 * values on the mesh's pattern selects the energy norm e^T K e / nact of the
 * normalised error over the active nodes, the quantity CG minimises.  The
 * matrix is read at each call. */
int fl_gnn_set_loss(fl_gnn net, const double* val);
int fl_gnn_get_weights(fl_gnn net, float* weights, int32_t count);
int fl_gnn_predict(fl_gnn net, const double* p1, const double* p2, const double* b, double* pred,
                   void* stream);
int fl_gnn_gradients(fl_gnn net, const double* p1, const double* p2, const double* b,
                     const double* target, const uint8_t* mask, int32_t nact, float* grad,
                     float* loss, void* stream);
int fl_gnn_train_step(fl_gnn net, const double* p1, const double* p2, const double* b,
                      const double* target, const uint8_t* mask, int32_t nact, float lr,
                      float* loss_dev, void* stream);

/* ------------------------------------------------ pressure projection -- */
/* P1 pressure and P1 velocity on one mesh handle (the P1-P1 configuration of
 * the projection method).  The divergence matrix ct_m is a block_csr_matrix
 * with blocks (1, dim): three device arrays of mesh-pattern values.  Vector
 * fields are vector_field%val(3, N) (x, y, z of a node adjacent). */

/* Second-order sparsity of the mesh's first-order pattern
 * (get_csr_sparsity_secondorder, femtools/Sparsity_Patterns_Meshes.F90:122-148
 * -> make_sparsity_transpose, femtools/Sparsity_Patterns.F90:87-148), built on
 * the GPU and bit-exact, as a pattern-only handle usable by fl_dev_petsc_solve,
 * fl_dev_csr_mult, fl_dev_apply_dirichlet and fl_gpu_sparsity_copy, and by the
 * row products below.  The mesh must outlive the returned handle. */
int fl_gpu_secondorder_register(fl_mesh mesh, fl_mesh* out);

/* Options of assemble_divergence_matrix_cg (assemble/Divergence_Matrix_CG.F90:
 * 67-375).  By parts, the surface loop (:312-366) runs over the nfaces surface
 * triangles: faces(3, nfaces) = face_global_nodes, face_ele(nfaces) = the
 * volume element of each face, bc_type(3, nfaces) = field_bc_type(dim, sele)
 * (0 none or strong Dirichlet, 1 weakdirichlet, 2 no_normal_flow, 3 internal,
 * 4 free_surface, 5 prescribed_normal_flow), bc_val(3, 3, nfaces) =
 * ele_val(field_bc, dim, sele) per face node (types 1 and 5 only; may be null
 * otherwise). */
typedef struct {
  int32_t integrate_by_parts;
  int32_t nfaces;
  int32_t index_base;
  int32_t pad;
  const int32_t* faces;
  const int32_t* face_ele;
  const int32_t* bc_type;
  const double* bc_val;
} fl_divergence_params;

/* Replaces assemble_divergence_matrix_cg for P1P1, single phase: ct_val[dim]
 * (mesh nnz each), ct_rhs (N, zeroed then the weak-Dirichlet / normal-flow
 * surface terms; may be null), div_mass_lumped and grad_mass_lumped (N; may
 * be null).  Device pointers; element contributions are summed in colour
 * order and are deterministic. */
int fl_dev_assemble_divergence_cg(fl_mesh mesh, const fl_divergence_params* params, double* const ct_val[3],
                                  double* ct_rhs, double* div_mass_lumped, double* grad_mass_lumped,
                                  void* stream);

/* Taylor-Hood pair: P2 velocity (the mesh) and P1 pressure on its vertices.
 * fl_gpu_rect_register builds make_sparsity(pressure mesh, velocity mesh)
 * (femtools/Sparsity_Patterns.F90:47-85) on the GPU: row v, a vertex of the
 * coordinate mesh, holds the P2 nodes of the elements containing v,
 * ascending; a pattern-only handle with one row per vertex.
 * fl_dev_assemble_divergence_p2p1 assembles the element terms of
 * assemble_divergence_matrix_cg (assemble/Divergence_Matrix_CG.F90:67-375)
 * for that pair into the three blocks of ct_m (shape_dshape, or
 * -dshape_shape by parts), each row summed in ascending element order;
 * quad_degree is the rule's degree (4 for P2).  The by-parts surface terms
 * are fl_dev_assemble_divergence_p2p1_faces.  Device pointers. */
int fl_gpu_rect_register(fl_mesh mesh, fl_mesh* out);
int fl_dev_assemble_divergence_p2p1(fl_mesh mesh, fl_mesh pattern, int32_t integrate_by_parts,
                                    int32_t quad_degree, double* const ct_val[3], void* stream);

/* The by-parts surface loop of assemble_divergence_matrix_cg
 * (assemble/Divergence_Matrix_CG.F90:312-366) for the same Taylor-Hood pair:
 * params->faces(3, nfaces) are the pressure (vertex) nodes of each surface
 * triangle, vfaces(6, nfaces) its P2 velocity nodes (face_global_nodes of the
 * velocity mesh in the triangle's local order: vertex 1, edge 12, vertex 2,
 * edge 13, edge 23, vertex 3), face_ele and bc_type as in
 * fl_divergence_params, and bc_val(3, 6, nfaces) the velocity bc per velocity
 * face node (types 1 and 5 only).  Adds into ct_val (the pattern's nnz each)
 * and subtracts from ct_rhs (pressure nodes, as the caller initialised it;
 * may be null), each pressure row's faces in ascending order; quad_degree
 * selects the triangle rule.  Device pointers. */
int fl_dev_assemble_divergence_p2p1_faces(fl_mesh mesh, fl_mesh pattern, const fl_divergence_params* params,
                                          const int32_t* vfaces, int32_t quad_degree, double* const ct_val[3],
                                          double* ct_rhs, void* stream);

/* The pattern of the Taylor-Hood cmc_m: get_csr_sparsity_secondorder(state,
 * p_mesh, u_mesh) (femtools/Sparsity_Patterns_Meshes.F90:122-148), i.e.
 * make_sparsity_transpose of the divergence pattern with itself (pressure
 * rows, pressure columns through the shared P2 velocity nodes), built on the
 * GPU as a pattern-only handle.  fl_dev_mult_div_vector_div_T on it forms
 * C_P^T diag(w) C with a and b on the pattern of fl_gpu_rect_register and w
 * per velocity node (assemble_masslumped_cmc, assemble/Assemble_CMC.F90:119-
 * 135, with the P2 lumped velocity mass); solves, SpMVs and Dirichlet
 * conditions run on it as on any pattern-only handle.  The pattern handle
 * must outlive it. */
int fl_gpu_rect_secondorder_register(fl_mesh pattern, fl_mesh* out);

/* compute_lumped_mass (femtools/FEFields.F90:161-214) of a P1 or P2 mesh with
 * unit density, as get_lumped_mass (femtools/State_Fields.F90:124-152) caches
 * it: the row sums of the consistent mass matrix (for P2, negative at the
 * vertices), each node's elements summed in ascending order. */
int fl_dev_lumped_mass(fl_mesh mesh, double* lumped_mass, void* stream);

/* mult_div_vector_div_T (femtools/Sparse_Matrices_Fields.F90:590-671):
 * out(i,j) = sum_k sum_dim a_dim(i,k) w(dim,k) b_dim(j,k) over the
 * second-order pattern `product`; a and b are ndim blocks on the parent
 * mesh's pattern, w is vector_field%val(ndim, N).  With a = ctp_m, b = ct_m
 * and w the inverse lumped mass it is assemble_masslumped_cmc
 * (assemble/Assemble_CMC.F90:119-135). */
int fl_dev_mult_div_vector_div_T(fl_mesh product, int32_t ndim, const double* const a_val[3], const double* w,
                                 const double* const b_val[3], double* out, void* stream);
/* mult_div_invscalar_div_T (femtools/Sparse_Matrices_Fields.F90:673-748):
 * out(i,j) = sum_k a(i,k) b(j,k) / s(k).  Every entry of a second-order
 * pattern has a common column, so every output entry is written at its own
 * position. */
int fl_dev_mult_div_invscalar_div_T(fl_mesh product, const double* a_val, const double* s_val,
                                    const double* b_val, double* out, void* stream);

/* assemble_kmk_matrix (assemble/Momentum_CG.F90:2707-2766): the P1-P1 pressure
 * stabilisation K^T M_l^-1 K / theta_pg over the second-order pattern, K the
 * pressure diffusion matrix with the elements' edge-length tensors
 * (0.5 dshape_tensor_dshape with h_bar = get_edge_lengths).  kt_val receives K
 * (mesh nnz; may be null). */
int fl_dev_assemble_kmk(fl_mesh mesh, fl_mesh product, double theta_pg, const double* p_masslump, double* kt_val,
                        double* kmk_val, void* stream);

/* assemble_masslumped_poisson_rhs (assemble/Momentum_CG.F90:2670-2705):
 * poisson_rhs = -C_P (M_l^-1 mom_rhs + u / (dt theta_pg)) + ct_rhs / (dt theta_pg);
 * mom_rhs and ct_rhs may be null (zero). */
int fl_dev_masslumped_poisson_rhs(fl_mesh mesh, const double* const ctp_val[3], const double* mom_rhs,
                                  const double* ct_rhs, const double* inverse_masslump, const double* velocity,
                                  double dt, double theta_pg, double* poisson_rhs, void* stream);
/* correct_masslumped_velocity (assemble/Momentum_CG.F90:2544-2575):
 * u += M_l^-1 C^T delta_p. */
int fl_dev_correct_masslumped_velocity(fl_mesh mesh, const double* const ct_val[3], const double* inverse_masslump,
                                       const double* delta_p, double* velocity, void* stream);
/* addto(matrix, other, scale) for two matrices on one pattern (add_kmk_matrix,
 * assemble/Momentum_CG.F90:2768-2777, is scale 1). */
int fl_dev_csr_addto(fl_mesh pattern, double* val, const double* other, double scale, void* stream);

/* Number of kernels this library launched on the calling process so far
 * (launch accounting for benchmarks). */
int64_t fl_kernel_launch_count(void);

/* Profiling hooks in the spirit of the reference's profiler keys
 * ("advection_diffusion_loop", Advection_Diffusion_CG.F90:574-600): when
 * enabled, the element loop of each assembly call on the handle is bracketed
 * by CUDA events on its stream, and fl_last_assembly_kernel_ms returns the
 * device time of that loop (all colours) for the last call. */
int fl_set_kernel_timing(fl_mesh mesh, int32_t on);
int fl_last_assembly_kernel_ms(fl_mesh mesh, float* ms);

#ifdef __cplusplus
}
#endif

#endif /* FLUIDITY_GB300_H */
