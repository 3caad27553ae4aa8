/* libsucem_gb300 -- C-ABI of the GB300 N1curl system-matrix and solve path.
 *
 * The reference (cemagg/sucem-fem) is Python; its FFI for this path is the
 * Python call into DOLFIN/FFC/scipy.  Each entry point below names the
 * reference call it replaces.  Conventions:
 *   - every function returns an int status: SUCEM_OK (0) or a negative
 *     SUCEM_ERR_* code; sucem_last_error() gives the message (per thread);
 *   - plain pointers and sizes only.  "device" pointers are CUDA device
 *     addresses on the device the space was uploaded to; "host" pointers are
 *     ordinary host memory; "stream" is a cudaStream_t (NULL = legacy stream);
 *   - the caller owns every buffer it passes; the library owns what sits
 *     behind a sucem_space handle and frees it in sucem_space_destroy;
 *   - handles are not thread safe; use one per thread or serialise calls.
 */
#ifndef SUCEM_GB300_H
#define SUCEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SUCEM_ABI_VERSION 1

#define SUCEM_OK 0
#define SUCEM_ERR_ARG -1       /* bad argument (ValueError in the Python layer) */
#define SUCEM_ERR_MEMORY -2    /* host or device allocation refused */
#define SUCEM_ERR_CUDA -3      /* a CUDA call failed */
#define SUCEM_ERR_STATE -4     /* call order (e.g. space not uploaded) */
#define SUCEM_ERR_NOCONV -5    /* iterative solve did not converge */
#define SUCEM_ERR_BREAKDOWN -6 /* Krylov breakdown / zero pivot / NaN */

typedef struct sucem_space sucem_space;

/* value dtypes of CSR arrays and vectors */
#define SUCEM_F32 0
#define SUCEM_F64 1
#define SUCEM_C64 2  /* interleaved complex float */
#define SUCEM_C128 3 /* interleaved complex double */

int sucem_version(void);
const char* sucem_last_error(void);
/* Number of kernels the library has launched since it was loaded (all
 * threads); used to report the kernel count of a timed region. */
long long sucem_launch_count(void);

/* Mesh + N1curl function space.  Replaces dolfin.FunctionSpace(mesh,
 * "Nedelec 1st kind H(curl)", order) and the sparsity pass of
 * dolfin.assemble (sucemfem/ProblemConfigurations/EMProblem.py:100-105,
 * sucemfem/SystemMatrices.py:54).  coords: nv*3 doubles; cells: nt*4
 * vertex ids (any vertex order; sorted internally as DOLFIN orders meshes);
 * order 1, 2, 3 or 4 (6, 20, 45, 84 DOFs per cell; orders 3 and 4 are the
 * degrees of functional_tests/test_EigenProblems.py:86,150).  Builds
 * entities, the DOF map (DOLFIN numbering for orders 1-2; k DOFs per edge,
 * k(k-1) per face, then the cell interiors for order k), the CSR pattern
 * and the row-gather tables (orders 1-2) or the per-cell CSR positions
 * (orders 3-4) on the host.  Point sources, field reconstruction, flux,
 * NTFF, EM functional and boundary interpolation take orders 1 and 2 and
 * return SUCEM_ERR_ARG on order-3/4 spaces. */
int sucem_space_create(const double* coords, int64_t nv, const int64_t* cells, int64_t nt,
                       int order, sucem_space** out);
void sucem_space_destroy(sucem_space* sp);

/* out[10] = {n_dofs (global_dimension, EMProblem.py:44-47), nnz, nv, nt,
 *            n_edges, n_faces, n_exterior_facets, n_boundary_dofs,
 *            longest_row, n_incidences} */
int sucem_space_sizes(const sucem_space* sp, int64_t* out);

#define SUCEM_COPY_INDPTR 0         /* int64[n+1] CSR row pointer */
#define SUCEM_COPY_INDICES 1        /* int32[nnz] CSR columns (sorted per row) */
#define SUCEM_COPY_CELL_DOFS 2      /* int32[nt*ndof] DOF map (dofmap().tabulate_dofs) */
#define SUCEM_COPY_BOUNDARY_DOFS 3  /* int32[n_boundary_dofs] PEC DOFs (essential.py:86-99) */
#define SUCEM_COPY_EDGES 4          /* int32[ne*2] */
#define SUCEM_COPY_FACES 5          /* int32[nf*3] */
#define SUCEM_COPY_CELLS 6          /* int32[nt*4] ordered cells */
#define SUCEM_COPY_EXT_MASK 7       /* uint8[nt] exterior-facet bit mask */
#define SUCEM_COPY_CELL_EDGES 8     /* int32[nt*6] cell -> edge ids (UFC local order) */
#define SUCEM_COPY_CELL_FACES 9     /* int32[nt*4] cell -> face ids (= facet numbering) */
#define SUCEM_COPY_DOF_XYZ 10       /* double[n*3] DOF locations (edge midpoint / face or cell
                                       centroid) */
#define SUCEM_COPY_BOUNDARY_DUAL 11 /* double[n_boundary_dofs*6] dual functional of each boundary
                                       DOF: point, tangent (DOF(u) = u(point).tangent) */
#define SUCEM_COPY_TASK_ENT 12     /* int32[n_tasks*32] assembly schedule: entity of each lane */
#define SUCEM_COPY_TASK_META 13    /* int32[n_tasks*4] first step block, steps per local entity
                                      index (8 bytes), flags (bit 0: faces; bits 8-23: the
                                      task's longest row, made odd) */
#define SUCEM_COPY_STEP_WORDS 14   /* uint32[n_step_blocks*(1+slot_planes)*32] step blocks */
#define SUCEM_COPY_ENTRY_PTR 15    /* int32[nnz+1] orders 3-4: first cell entry of each CSR entry
                                      (empty for orders 1-2) */
#define SUCEM_COPY_ENTRY_SRC 16    /* int32[nt*ndof*ndof] orders 3-4: the cell entries
                                      (c*ndof + a)*ndof + b summed into each CSR entry, in
                                      ascending cell order */
#define SUCEM_COPY_ENTRY_PERM 17   /* int32[nnz] orders 3-4: the CSR entry of each assembly
                                      thread (each row's entries by list length) */
int sucem_space_copy(const sucem_space* sp, int what, void* host_dst);

/* Sizes of the order-1/2 assembly schedule (the kernel's work plan; no
 * reference counterpart, exposed so that tests can check it on the host):
 * out[4] = {n_tasks, n_tasks_interior, n_step_blocks, slot_planes}. */
int sucem_space_schedule_sizes(const sucem_space* sp, int64_t* out);

/* Copies the space to CUDA device `device` (idempotent). */
int sucem_space_upload(sucem_space* sp, int device);

#define SUCEM_DEV_INDPTR 0          /* int32[n+1] */
#define SUCEM_DEV_INDICES 1         /* int32[nnz] */
#define SUCEM_DEV_CELL_DOFS 2       /* int32[nt*ndof] */
#define SUCEM_DEV_BOUNDARY_DOFS 3   /* int32[n_boundary_dofs] */
int sucem_space_device_ptr(const sucem_space* sp, int what, void** out);

/* Assembly of the interior forms and the ABC form into CSR values on the
 * space's pattern.  Replaces dolfin.assemble of
 *   S   = dot(curl(v), curl(u))/mu_r*dx   (sucemfem/Forms.py:79-85)
 *   M=T = eps_r*inner(v, u)*dx            (sucemfem/Forms.py:71-77)
 *   S_0 = inner(cross(n,v), cross(n,u))*ds over every exterior facet
 *         (sucemfem/BoundaryConditions/ABC.py:56-57)
 * as called from SystemMatrices.calc_system_matrices
 * (sucemfem/SystemMatrices.py:46-58).  real_bytes = 4 (float) or 8
 * (double) selects the precision of the coefficients and outputs.
 * eps_r, mu_r_inv: device arrays of nt values (NULL = 1, the material
 * defaults of sucemfem/Materials.py:31).  S, T, B: device arrays of nnz
 * values; any may be NULL to skip that matrix.  Orders 1-2 write every
 * value once in a fixed summation order; orders 3-4 zero the outputs and
 * add the cells' contributions atomically (summation order not fixed). */
int sucem_assemble(const sucem_space* sp, int real_bytes, const void* eps_r,
                   const void* mu_r_inv, void* S, void* T, void* B, void* stream);

/* Fused driven-problem matrix A = S - k0^2 T + 1j*k0*B written as
 * interleaved complex (complex64 for real_bytes 4, complex128 for 8) on the
 * full cell pattern.  Replaces DrivenProblemABC.get_LHS_matrix
 * (sucemfem/ProblemConfigurations/EMDrivenProblem.py:67-72) without the
 * exact-zero compaction scipy's sparse arithmetic performs. */
int sucem_assemble_helmholtz(const sucem_space* sp, int real_bytes, const void* eps_r,
                             const void* mu_r_inv, double k0, void* A, void* stream);

/* Same as sucem_assemble with host buffers: copies in, assembles, copies
 * back (synchronous).  The end-to-end form of dolfin.assemble. */
int sucem_assemble_host(const sucem_space* sp, int real_bytes, const void* eps_r_host,
                        const void* mu_r_inv_host, void* S_host, void* T_host, void* B_host);

/* Essential (PEC) rows: zero each listed row of a value array on the
 * space's pattern and set its diagonal to 1, columns untouched.  Replaces
 * dolfin.DirichletBC(...).apply(A) as called by
 * EssentialBoundaryCondition.get_essential_application_func
 * (sucemfem/BoundaryConditions/essential.py:65-81).  dtype F32 or F64;
 * rows: device int32[nrows]. */
int sucem_apply_essential(const sucem_space* sp, int dtype, void* vals, const int32_t* rows,
                          int64_t nrows, void* stream);

/* y = A x on the space's pattern (device arrays).  Replaces the matrix-vector
 * products M*x of sucemfem/ProblemConfigurations/EMVectorWaveEigenproblem.py:86,98
 * and A*x of calculate_residual (sucemfem/Utilities/LinalgSolvers.py:297-305). */
int sucem_spmv(const sucem_space* sp, int dtype, const void* vals, const void* x, void* y,
               void* stream);

/* out = a*X + b*Y (+ j*c*Z when complex_out) elementwise over m values
 * (device arrays, NULL operands skipped).  Replaces the sparse linear
 * combinations S - sigma*M (EMVectorWaveEigenproblem.py:76) and
 * S - k0**2*M + 1j*k0*S_0 (EMDrivenProblem.py:72) on a shared pattern. */
int sucem_combine(int64_t m, int real_bytes, double a, const void* X, double b, const void* Y,
                  double c, const void* Z, void* out, int complex_out, void* stream);

/* Drop exact (complex) zeros from a complex CSR on the space's pattern, as
 * scipy's sparse binary operators do for the result of get_LHS_matrix
 * (EMDrivenProblem.py:72).  Two steps: count (writes out_indptr[n+1];
 * work = device int32[n]) then fill (out_indices, out_vals sized
 * out_indptr[n]). */
int sucem_compact_count(const sucem_space* sp, int dtype, const void* vals, int32_t* out_indptr,
                        int32_t* work, void* stream);
int sucem_compact_fill(const sucem_space* sp, int dtype, const void* vals,
                       const int32_t* out_indptr, int32_t* out_indices, void* out_vals,
                       void* stream);

/* Allocation-free form of sucem_compact_count; no counterpart in the
 * reference.  For callers that cannot allocate device memory when they need
 * the compaction (for example a serving loop that reserved its whole HBM
 * budget for resident problems, or a host whose device memory belongs to
 * another allocator): the per-row count scratch is a fixed array inside the
 * library (4 MiB, held on every GPU that loads the library until exit), so
 * no work buffer is passed and nothing is allocated.  Limit: at most 2^20
 * rows; larger matrices get SUCEM_ERR_ARG with a message.  The first call on
 * a device looks up the array's device address (make that first call before
 * any stream capture).  Every call shares the one array: calls that overlap
 * on the GPU (other streams, other threads) race and must be serialised.
 * The device address looked up on the first call is cached for the life of
 * the process; it is not refreshed after cudaDeviceReset, so do not call
 * this entry point on a device that the process has reset. */
int sucem_compact_count_noalloc(const sucem_space* sp, int dtype, const void* vals,
                                int32_t* out_indptr, void* stream);

/* Point current sources: locate each point (lowest-index cell whose closure
 * contains it) and evaluate N_i(p) . value for the ndof basis functions of
 * that cell.  Replaces calc_pointsource_contrib
 * (sucemfem/Sources/point_source.py:49-94).  Device arrays: pts double
 * [npts*3]; values complex128 [npts*3] (interleaved); cells_out int32
 * [npts] (0x7f7f7f7f when the point is outside the mesh); contrib
 * complex128 [npts*ndof]. */
int sucem_point_sources(const sucem_space* sp, const double* pts, const double* values, int npts,
                        int32_t* cells_out, double* contrib, void* stream);

/* The field E(p) = sum_i x_i N_i(p) at points.  Replaces
 * Reconstruct.reconstruct_points (sucemfem/PostProcessing/
 * PostProcessing.py:27-60).  Points are located as for the point sources
 * (lowest-index cell whose closure contains the point).  Device arrays: x
 * the DOF vector (dtype SUCEM_C64 or SUCEM_C128, interleaved complex); pts
 * double[npts*3]; cells_out int32[npts] (0x7f7f7f7f for a point outside the
 * mesh); E complex128[npts*3] (NaN for a point outside the mesh). */
int sucem_reconstruct_points(const sucem_space* sp, int dtype, const void* x, const double* pts,
                             int npts, int32_t* cells_out, double* E, void* stream);

/* Real power flux through the whole mesh boundary, replacing
 * SurfaceFlux.calc_flux (sucemfem/PostProcessing/power_flux.py:11-60):
 *   (1/(k0 Z0)) * int n . (E_r x (-curl E_i / mu_r) + E_i x (curl E_r / mu_r)) ds
 * over every exterior facet with the outward normal n (a 9-point facet rule,
 * exact for orders 1 and 2).  Device arrays: x (SUCEM_C64 or SUCEM_C128);
 * mu_r double per cell or NULL (1); part double[nt] scratch (per-cell
 * contributions); out double[1].  The sum is taken in a fixed order, so
 * repeated calls give identical results. */
int sucem_surface_flux(const sucem_space* sp, int dtype, const void* x, double k0,
                       const double* mu_r, double* part, double* out, void* stream);

/* Surface near-to-far-field transform, replacing NTFF.calc_pt
 * (sucemfem/PostProcessing/surface_ntff.py:29-155): equivalent currents
 * J = n x H (H = j curl E / (k0 Z0)) and M = -n x E on every exterior facet,
 * radiated to the directions (theta[d], phi[d]) (radians, device arrays):
 *   N = int J e^{j k0 r'.r_hat} ds,  L = int M e^{j k0 r'.r_hat} ds,
 *   E_theta = -r_fac (L_phi + Z0 N_theta),  E_phi = r_fac (L_theta - Z0 N_phi),
 *   r_fac = j k0 e^{-j k0} / (4 pi)  (far field normalised to radius 1),
 * with the 9-point collapsed Gauss-Jacobi facet rule.  out: device double
 * [ndir*12] = per direction E_theta, E_phi, L_theta, L_phi, N_theta, N_phi
 * (complex, interleaved); each direction is summed in a fixed order.  The
 * per-point scratch lives in the space handle (allocated on the first
 * call): calls on one space must not overlap on the GPU. */
int sucem_ntff(const sucem_space* sp, int dtype, const void* x, double k0, int ndir,
               const double* theta, const double* phi, double* out, void* stream);

/* The EM functional of CalcEMFunctional.calc_functional
 * (sucemfem/PostProcessing/PostProcessing.py:62-173):
 *   I = sum over the marked cells of
 *       int curl E . curl g / mu_r - k0^2 eps_r E . g dx   (bilinear)
 * evaluated element by element (exact: the reference element tensors).
 * Device arrays: E, g complex128[n]; eps_r, mu_r_inv double per cell or
 * NULL (1); cell_mask uint8 per cell or NULL (all cells); part
 * double[2*nt] scratch; out double[2] (fixed-order sum). */
int sucem_em_functional(const sucem_space* sp, const double* E, const double* g, double k0,
                        const double* eps_r, const double* mu_r_inv, const uint8_t* cell_mask,
                        double* part, double* out, void* stream);

/* Cells with an edge on the boundary (sucemfem/Geometry.py:76-90
 * BoundaryEdgeCells), host array uint8[nt]. */
int sucem_boundary_edge_cells(const sucem_space* sp, uint8_t* mask);

/* Plane-wave testing functions interpolated onto the boundary DOFs, the
 * SurfaceInterpolant of TransformTestingExpression
 * (sucemfem/PostProcessing/variational_ntff.py:31-66,
 * sucemfem/Interpolation/Interpolation.py:71-82): for wave w and boundary
 * DOF d (dual functional point p, tangent t)
 *   g[w*n + d] = j (t . cf_w) e^{j k0 rhat_w . p}
 * Device arrays: rhat, cf double[npw*3]; g complex128[npw*n]; only the
 * boundary DOFs are written (the caller zeroes the rest). */
int sucem_plane_wave_dofs(const sucem_space* sp, int npw, const double* rhat, const double* cf,
                          double k0, double* g, void* stream);

/* ---- vectors and general CSR (device arrays) ----
 * The Krylov / refinement building blocks behind solve_sparse_system and the
 * solver classes of sucemfem/Utilities/LinalgSolvers.py:239-322.
 * spmv_csr: y = A x for any CSR with int32 indices.
 * axpby: y = a*x + b*y, a and b complex (imaginary parts ignored for real
 * dtypes; x may be NULL for y = b*y).
 * dot: out[0..1] (device, double re/im) = sum conj(x)*y (conj=1) or x*y,
 * accumulated in double in a fixed order; work = device scratch of
 * sucem_vec_dot_work_bytes() bytes.
 * convert: count reals between float and double arrays. */
int sucem_spmv_csr(int64_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                   int dtype, const void* vals, const void* x, void* y, void* stream);
int sucem_vec_axpby(int64_t n, int dtype, double ar, double ai, const void* x, double br,
                    double bi, void* y, void* stream);
int64_t sucem_vec_dot_work_bytes(void);
int sucem_vec_dot(int64_t n, int dtype, const void* x, const void* y, int conj, void* work,
                  double* out, void* stream);
int sucem_vec_convert(int64_t count, int dst_real_bytes, void* dst, int src_real_bytes,
                      const void* src, void* stream);
/* Block Gram-Schmidt step of FGMRES (the orthogonalisation inside
 * GMRESSolver, sucemfem/Utilities/LinalgSolvers.py:251-260, scipy's gmres):
 * w is made orthogonal to the k rows V_i of V (leading dimension ldv
 * elements) by classical Gram-Schmidt with one reorthogonalisation, all on
 * the device; h[0:k] (complex as double pairs, real parts for F64) receive
 * the summed coefficients conj(V_i)·w of both passes and h[k] the squared
 * norm of the result (real part), so one copy to the host serves a whole
 * Arnoldi step.  dtype F64 or C128; 0 <= k <= 63; work holds
 * sucem_vec_gs_work_bytes(k) bytes; h is device memory of (k + 1) pairs. */
int64_t sucem_vec_gs_work_bytes(int k);
int sucem_vec_gs(int64_t n, int dtype, const void* V, int64_t ldv, int k, void* w, void* work,
                 double* h, void* stream);

/* Segmented (batched) double vectors for the batched Lanczos of
 * DefaultEigenSolver.solve_problem (EMVectorWaveEigenproblem.py:61-105,
 * ARPACK's inner products and updates): independent problems are stacked,
 * segment s covering [seg_ptr[s], seg_ptr[s+1]).
 * seg_dot: out[j*nseg + s] = X_j . y over segment s, X_j = X + j*ldx.
 * seg_axpy: y_i = b[s] y_i + sum_j a[j*nseg + s] X_j,i (b NULL = 1);
 * seg_of: int32[n] segment of every entry. */
int sucem_seg_dot(int nseg, const int64_t* seg_ptr, const double* X, int64_t ldx, int nvec,
                  const double* y, double* out, void* stream);
/* dst[i] = src[idx[i]] (elements of 4, 8 or 16 bytes): extracts the values
 * of a sub-matrix (e.g. the PEC-free DOFs) from a CSR value array. */
int sucem_gather(int64_t m, int elem_bytes, const int64_t* idx, const void* src, void* dst,
                 void* stream);
int sucem_seg_axpy(int nseg, const int64_t* seg_ptr, int64_t n, const int32_t* seg_of,
                   const double* X, int64_t ldx, int nvec, const double* a, const double* b,
                   double* y, void* stream);

/* ---- multifrontal sparse LU (GPU) ----
 * Replaces the reference's direct solves: dolfin.LUSolver(S - sigma*M)
 * (sucemfem/ProblemConfigurations/EMVectorWaveEigenproblem.py:76-85),
 * UMFPACKSolver / spsolve (sucemfem/Utilities/LinalgSolvers.py:262-277) and,
 * used as a preconditioner, spilu (LinalgSolvers.py:118-121).
 * analyse: host CSR pattern with symmetric structure (sorted columns) and
 * n*3 DOF coordinates (NULL: breadth-first-distance pseudo-coordinates of
 * the matrix graph); builds a nested-dissection ordering and the front
 * structure on the host.  factor: device values in CSR order (dtype
 * SUCEM_F32/F64/C64/C128), no pivoting; pivots below pivot_tol*max|a_ij|
 * are replaced (static pivoting, count via sucem_lu_perturbed).  solve:
 * device b, x of n values in the factor's dtype or, for a single-precision
 * factor, its double-precision twin (conversion on the fly). */
typedef struct sucem_lu sucem_lu;
int sucem_lu_analyse(int64_t n, const int32_t* indptr, const int32_t* indices, const double* xyz,
                     int leaf_size, sucem_lu** out);
/* Same analysis with the element-based nested dissection (preferred for FEM
 * matrices): cell_dofs int32[nt*ndof_cell] (-1 for DOFs not in the matrix),
 * cell_xyz double[nt*3] cell centroids.  Separators are interface surfaces
 * between bisected cell sets. */
int sucem_lu_analyse_cells(int64_t n, const int32_t* indptr, const int32_t* indices, int64_t nt,
                           int ndof_cell, const int32_t* cell_dofs, const double* cell_xyz,
                           int leaf_size, sucem_lu** out);
void sucem_lu_destroy(sucem_lu* lu);
/* out[7] = {n, nnz, tree nodes, tree levels, front arena entries, factor
 *           multiply-adds, largest front} */
int sucem_lu_info(const sucem_lu* lu, double* out);
int sucem_lu_copy_perm(const sucem_lu* lu, int64_t* perm);
/* The assembly tree, for inspection: out[3*i .. 3*i+2] = {level (leaves 0),
 * pivots k, front size f} of tree node i (i < tree nodes of sucem_lu_info).
 * No reference counterpart (the reference's direct solve is a library
 * call). */
int sucem_lu_fronts(const sucem_lu* lu, int64_t* out);
int sucem_lu_factor(sucem_lu* lu, int dtype, const void* vals, double pivot_tol, void* stream);
int sucem_lu_solve(sucem_lu* lu, int io_dtype, const void* b, void* x, void* stream);
int sucem_lu_perturbed(sucem_lu* lu);
/* Waits for the last factorisation and reports whether it can be used:
 * SUCEM_OK, or SUCEM_ERR_STATE when it was not factored or when a bounded
 * wait of its tensor-core update gave up (the factor is then invalid, and
 * sucem_lu_solve refuses it with the same error).  No reference counterpart:
 * dolfin.LUSolver / UMFPACK report no such device-side failure
 * (EMVectorWaveEigenproblem.py:76-79, LinalgSolvers.py:262-277). */
int sucem_lu_status(sucem_lu* lu);
/* Test hook, no reference counterpart: marks the last factorisation as if a
 * bounded wait of its tensor-core update had given up (a host write of the
 * device flag; no kernel is made to fail), so that tests can check that
 * sucem_lu_status and sucem_lu_solve refuse the factor. */
int sucem_lu_inject_timeout(sucem_lu* lu);
/* Tensor-core Schur-update launches of the last complex64 factorisation
 * (waits for them): out[3] = {launches, summed event-timed duration in ms,
 * algorithmic flops (8 per complex multiply-add)}.  No reference
 * counterpart (measurement hook). */
int sucem_lu_kernel_stats(sucem_lu* lu, double* out);
/* Preconditioned BiCGStab on the device, every scalar kept in device
 * memory.  Replaces BiCGStabSolver (sucemfem/Utilities/LinalgSolvers.py:
 * 239-248: scipy.sparse.linalg.bicgstab with the preconditioner of :107-127).
 * A: CSR of n rows (int32 indptr[n+1], indices; values of dtype SUCEM_C64 or
 * SUCEM_C128); b, x: device vectors of that dtype (x holds the initial
 * guess on entry, the solution on exit).  precond: 0 none, 1 diagonal
 * (inverse of A's diagonal), 2 the factorisation `lu` (sucem_lu_solve).
 * Stops at ||b - A x|| <= tol ||b|| or after maxit iterations.  Without an
 * LU preconditioner `batch` iterations are captured once into a CUDA graph
 * and replayed; the host reads one status word per batch (with LU: per
 * iteration).  work: device buffer of sucem_bicgstab_work_bytes(n, dtype)
 * bytes.  info[4] = {iterations, ||r||/||b|| (recurrence residual),
 * status (1 converged, 2 iteration limit, -1 breakdown rho = 0,
 * -2 breakdown omega = 0), host synchronisations}. */
int64_t sucem_bicgstab_work_bytes(int64_t n, int dtype);
int sucem_bicgstab(int64_t n, const int32_t* indptr, const int32_t* indices, int dtype,
                   const void* vals, const void* b, void* x, int precond, sucem_lu* lu,
                   double tol, int maxit, int batch, void* work, int64_t work_bytes, double* info,
                   void* stream);

/* Plan parameters of the single-precision factorisation (tensor-core path),
 * 0 = default: the super-panel width (a positive multiple of 64; default
 * 512) and the smallest pivot block for which a level of two or more
 * fronts applies its 64-column panel updates on the tensor cores (default
 * 64).  The device state is rebuilt at the next sucem_lu_factor.  Used by
 * the autotuner (sucemfem/autotune.py).  No reference counterpart
 * (dolfin.LUSolver / UMFPACK take no such parameters). */
int sucem_lu_configure(sucem_lu* lu, int superpanel, int panel_min_k);

/* Self-test of the device-side failure detection: one thread of a one-block
 * kernel waits, with the tensor-core kernel's bounded mbarrier wait limited
 * to `polls` polls, for a barrier phase nothing completes; *gave_up = 1
 * when the wait ran out and the kernel returned (the expected outcome; the
 * CUDA context stays usable).  Synchronous on the default stream.  No
 * reference counterpart (the reference has no device code). */
int sucem_selftest_bounded_wait(int polls, int* gave_up);

#ifdef __cplusplus
}
#endif

#endif /* SUCEM_GB300_H */
