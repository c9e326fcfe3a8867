/*
 * lymph3d_gpu.h -- C ABI of the GB300 PolyDG elastodynamics hot path.
 *
 * This is the drop-in boundary for the matrix-free solver module of LYMPH3D
 * (src/matrix_free.f90).  Every entry point below replaces one subroutine the
 * Fortran driver src/Lymph3D.f90 calls; the citation next to each declaration
 * names the reference interface it stands for.  All arguments are plain C
 * types and pointers; no torch type or C++ type crosses this boundary.  Data
 * pointers are host pointers, with one exception: lymph_error_l2_noalloc
 * takes device pointers to the caller's own device arrays.  Everything else
 * in device memory, the streams and the kernels live behind the opaque
 * context handle.
 *
 * Conventions
 *  - Every function returns an int status: LYMPH_OK (0) or a code from the
 *    reference's Poly_exit_codes module (src/Poly_global.f90:130-173), or one
 *    of the LYMPH_ERR_* codes this library adds.  A failed call leaves a
 *    one-line explanation in lymph_last_error().  Nothing calls exit/stop.
 *  - Indices are 0-based (the Fortran side subtracts 1 once when flattening).
 *  - Degrees of freedom of a polyhedron are ordered component-major:
 *    dof = i*Np + m  (component i in 0..2, basis function m in 0..Np-1), the
 *    reference's row = (i-1)*Np + m (src/matrix_free.f90:240-256).
 *  - One context per host thread; calls are stream-ordered on the context's
 *    own stream and synchronous at return.
 *  - A polyhedron is a set of tetrahedra (tet_poly).  When every polyhedron
 *    holds one tetrahedron the operator is exactly the reference's per-tet
 *    operator; with agglomeration, volume integrals are summed over the
 *    sub-tetrahedra and only faces between different polyhedra (or on the
 *    boundary) carry face terms, the rule src/matrix_free.f90:290-309 applies.
 */
#ifndef LYMPH3D_GPU_H
#define LYMPH3D_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LYMPH_OK                       0
#define LYMPH_EXIT_INSTAB              2   /* NaN/Inf in the state (Poly_exit_codes EXIT_INSTAB) */
#define LYMPH_EXIT_SETUP               4   /* inconsistent mesh / parameters (EXIT_SETUP) */
#define LYMPH_EXIT_SINGULARMTX         5   /* mass matrix not SPD (EXIT_SINGULARMTX; cholesky stop) */
#define LYMPH_EXIT_ELEM_ORIENT        11   /* tetrahedron with det J <= 0 (EXIT_ELEM_ORIENT) */
#define LYMPH_EXIT_NEIGHBOUR_EL_ERROR 18   /* face neighbour table inconsistent (EXIT_NEIGHBOUR_EL_ERROR) */
#define LYMPH_ERR_INVALID            100   /* bad argument */
#define LYMPH_ERR_CUDA               101   /* CUDA runtime error */
#define LYMPH_ERR_OOM                102   /* device allocation failed */
#define LYMPH_ERR_ORDER              103   /* call made before its prerequisite */
#define LYMPH_ERR_TIMEOUT            104   /* a bounded device-side wait expired */
#define LYMPH_ERR_INDEX              105   /* device-side index check failed */

/* ---- boundary markers in lymph_mesh_desc.neigh (BC_DIRI / BC_NEUM /
 *      BC_ABSO, src/Poly_global.f90:420-422) ----------------------------- */
#define LYMPH_BC_DIRI (-1)
#define LYMPH_BC_NEUM (-2)
/* Absorbing face: no stiffness or load term (traction-free like a Neumann
 * face), plus the damping block of MAKE_DAMPING_FACE
 * (src/assemble_element.f90:666-731) on its polyhedron,
 *   D_P[(i,m),(j,n)] = sum_q w_q |face| phi_m phi_n (c_t (t1_i t1_j + t2_i t2_j) + c_n n_i n_j),
 * with the first-order impedances c_t = rho c_s = sqrt(rho mu) and
 * c_n = rho c_p = sqrt(rho (lambda + 2 mu)) of the face's tetrahedron (the
 * reference's c1, c2, c3; its matrix-free path leaves the call commented
 * out, src/matrix_free.f90:279-287).  The leapfrog step then solves
 *   (M + dt/2 D) u^{n+1} = dt^2 (F - K u^n) + 2 M u^n - (M - dt/2 D) u^{n-1}
 * on polyhedra with absorbing faces, and the first step subtracts D v^0 from
 * the load. */
#define LYMPH_BC_ABSO (-3)

/* ---- precision of the operator apply ----------------------------------- */
#define LYMPH_FP64   0   /* every operation in FP64 (the plain path) */
#define LYMPH_MIXED  1   /* operator blocks and their mat-vec in FP32, FP32
                            accumulation; every block assembled on the tensor
                            cores (kind::tf32, FP32-accurate split products);
                            geometry, mass matrices, mass inverse, time update
                            and error norms in FP64 */
#define LYMPH_MIXED_MF 2  /* FP32 self blocks (assembled on the tensor cores,
                            as for LYMPH_MIXED); the neighbour terms evaluated
                            matrix-free in FP32 at every step from the face
                            quadrature (Q's field and gradient at P's
                            quadrature points, tested against P's basis), so no
                            neighbour block is stored or read; the triangle
                            rule is exact to degree 2p with fewer nodes than
                            the reference's (lymph_mf_face_rule); FP32
                            accumulation, FP64 combine, mass inverse, update
                            and error norms. */

/* ---- state slots (the driver's arrays, src/Lymph3D.f90:237-239) --------- */
#define LYMPH_SLOT_U0   0   /* u0_loc: u^{n-1} (u^0 before the first step)   */
#define LYMPH_SLOT_UN   1   /* un_loc: u^n                                   */
#define LYMPH_SLOT_V0   2   /* v0_loc: initial velocity coefficients         */
#define LYMPH_SLOT_UEX  3   /* modal coefficients of the exact solution      */
#define LYMPH_NUM_SLOTS 4

/* ---- host array layouts for get/set ------------------------------------ */
#define LYMPH_LAYOUT_POLY_MAJOR 0  /* C array [n_poly][3*Np]                */
#define LYMPH_LAYOUT_FORTRAN    1  /* reference u(ie, k): column-major with the
                                      polyhedron index fastest, i.e. the C
                                      array [3*Np][n_poly]                    */

/* ---- RHS selector and data-function ids (procedure arguments of
 *      MAKE_RHS_FREE / COMPUTE_MODAL_COEFFICIENTS_FREE become ids) -------- */
#define LYMPH_RHS_STAT 0         /* rhs_stat_loc                              */
#define LYMPH_RHS_DYN  1         /* rhs_dyn_loc (scaled by time_function(t))   */

#define LYMPH_F_NULL   0         /* f_null          problem_data_and_properties.f90:72-82 */
#define LYMPH_F_TIME   1         /* f_time                                 :48-70  */
#define LYMPH_F_STAT   2         /* f (static manufactured forcing)        :26-45  */

#define LYMPH_GD_NULL  0         /* gd_null   :84-92   */
#define LYMPH_GD       1         /* gd        :130-154 */
#define LYMPH_GD_STAT  2         /* gd_stat   :106-114 */

#define LYMPH_GN_NULL  0         /* gn_null   :94-104  */
#define LYMPH_GN       1         /* gn        :186-242 */
#define LYMPH_GN_STAT  2         /* gn_stat   :116-128 */

#define LYMPH_FUN_IC_DISPLACEMENT 0  /* ic_displacement :281-290 (zero) */
#define LYMPH_FUN_IC_VELOCITY     1  /* ic_velocity     :292-301        */
#define LYMPH_FUN_UEX             2  /* uex             :245-254        */
#define LYMPH_FUN_UEX_STAT        3  /* uex_stat        :257-264 (zero) */

/* ---- operator block selector for lymph_get_blocks ----------------------- */
#define LYMPH_BLOCKS_K    0   /* stiffness blocks K_loc (K_loc(ie,1:5,:,:))   */
#define LYMPH_BLOCKS_ADG  1   /* DG-norm blocks A_dg_loc                      */

typedef struct lymph_ctx lymph_ctx;

/* Flattened mesh: the parts of Mesh_Structure / Element / Polyhedron
 * (src/Poly_mesh.f90:13-104) the hot path reads.  Geometry (Jacobians,
 * normals, areas, bounding boxes, diameters) is derived on the device from
 * these arrays, as src/Poly_ref_mappings.f90:18-75 and
 * src/MAKE_PARTITION_AND_MPI_FILES.f90:1429-1580 derive it. */
typedef struct lymph_mesh_desc {
    int32_t n_node;
    int32_t n_tet;
    int32_t n_poly;
    int32_t n_mat;
    const double*  coords;    /* [n_node][3]                                  */
    const int32_t* tet_vert;  /* [n_tet][4] node ids (Elem_loc%vert)          */
    const int32_t* tet_poly;  /* [n_tet] polyhedron id (elem_in_poly)          */
    const int32_t* tet_mat;   /* [n_tet] material id (Elem_loc%mat_prop)       */
    const int32_t* neigh;     /* [n_tet][4] tet across face f, or LYMPH_BC_DIRI /
                                 LYMPH_BC_NEUM / LYMPH_BC_ABSO (neigh_el(f,2)); face f joins
                                 vertices {1,2,3},{1,2,4},{2,3,4},{3,1,4}
                                 (1-based, MAKE_PARTITION_AND_MPI_FILES.f90:1087-1096) */
    const int32_t* fun_tag;   /* [n_tet][4] boundary space-function tag
                                 (neigh_el(f,5)); may be NULL (all 1)          */
    const double*  mat;       /* [n_mat][3] rho, lambda, mu (prop_mat(:,1:3))  */
} lymph_mesh_desc;

typedef struct lymph_params {
    int32_t degree;     /* polynomial degree p, 1..6 (Elem_loc%Degree)        */
    int32_t precision;  /* LYMPH_FP64, LYMPH_MIXED or LYMPH_MIXED_MF          */
    double  alpha;      /* penalty constant (set_properties: 10)              */
    double  theta;      /* -1 SIPG, 0 IIPG, 1 NIPG (set_properties: -1)       */
    double  dt;         /* time step (Poly.input TIMESTEP)                    */
} lymph_params;

/* Library version (major*10000 + minor*100 + patch). */
int lymph_version(void);

/* Last error message of the calling thread ("" if none). */
const char* lymph_last_error(void);

/* Copies the mesh to the device, derives geometry and the block pattern.
 * Replaces the flattening of Mesh_Structure the driver does before
 * src/Lymph3D.f90:262 (no counterpart subroutine: the reference passes the
 * derived type).  Keeps no host pointer. */
int lymph_create(const lymph_mesh_desc* mesh, const lymph_params* prm, lymph_ctx** out);

/* Frees every device resource of the context. */
int lymph_destroy(lymph_ctx* ctx);

/* Problem sizes: Np, number of polyhedra, number of operator blocks (self +
 * neighbour blocks), number of face-sides carrying face terms. */
int lymph_sizes(const lymph_ctx* ctx, int32_t* Np, int32_t* n_poly, int64_t* n_blocks, int64_t* n_face_sides);

/* MAKE_MATRICES_FREE (src/matrix_free.f90:27-464) followed by the Cholesky
 * factorisation of the mass matrices (src/Lymph3D.f90:264-271): assembles
 * K_loc, M_loc, M_modal_loc and their factors on the device (the FP32
 * blocks of the mixed precisions on the tensor cores). */
int lymph_make_matrices(lymph_ctx* ctx);

/* MAKE_RHS_FREE (src/matrix_free.f90:467-843): which = LYMPH_RHS_STAT or
 * LYMPH_RHS_DYN; the three procedure arguments become ids. */
int lymph_make_rhs(lymph_ctx* ctx, int which, int forcing_id, int dirichlet_id, int neumann_id);

/* COMPUTE_MODAL_COEFFICIENTS_FREE (src/matrix_free.f90:847-997): L2
 * projection of the data function fun_id into state slot `slot`, then the
 * slot is multiplied by `scale` (the driver's time_function(t) scaling,
 * src/Lymph3D.f90:459-466; pass 1.0 for none). */
int lymph_modal_project(lymph_ctx* ctx, int fun_id, int slot, double scale);

/* FIRST_TIME_STEP_MATRIX_FREE (src/matrix_free.f90:1100-1227):
 * UN <- U0 + dt V0 + dt^2/2 M^-1 (F_stat + F_dyn g(t) - K U0). */
int lymph_first_step(lymph_ctx* ctx, double t);

/* TIME_STEP_MATRIX_FREE (src/matrix_free.f90:1230-1385) plus the driver's
 * array rotation (src/Lymph3D.f90:393-397): computes
 * u^{n+1} = dt^2 M^-1 (F_stat + F_dyn g(t) - K u^n) + 2 u^n - u^{n-1},
 * then U0 <- u^n, UN <- u^{n+1}.  The neighbour coefficients the reference
 * receives through MPI_EXCHANGE_DOF (src/exchange_data.f90:153-258) are
 * gathered on the device. */
int lymph_step(lymph_ctx* ctx, double t);
/* TIME_STEP_MATRIX_FREE with the reference's host arrays (src/matrix_free.f90
 * :1230-1385, called at Lymph3D.f90:393 with the copies of :396-397 around
 * it): u0 = u^{n-1} and un = u^n go up, one leapfrog step at time t runs,
 * and usol = u^{n+1} comes back, in the given layout (LYMPH_LAYOUT_FORTRAN:
 * the reference's u(ie, k)).  The same values as lymph_set_state(U0, u0),
 * lymph_set_state(UN, un), lymph_step(t), lymph_get_state(UN, usol), with
 * the two uploads on separate streams and one synchronisation.  Afterwards
 * the context holds U0 = u^n and UN = u^{n+1}. */
int lymph_time_step_host(lymph_ctx* ctx, double t, const double* u0, const double* un, double* usol, int layout);

/* The two steps above with the time-function value g supplied by the caller
 * instead of sin(sqrt(2) pi t) (problem_data_and_properties.f90:14-23), for
 * sources with another time dependence (e.g. a Ricker wavelet). */
int lymph_first_step_g(lymph_ctx* ctx, double g);
int lymph_step_g(lymph_ctx* ctx, double g);

/* The time loop of src/Lymph3D.f90:389-418: while (*t_inout <= stop_time)
 * { step(*t_inout); *t_inout += dt; }, at most max_steps steps
 * (max_steps < 0: no cap).  The time function values are computed on the
 * host with the reference's floating-point accumulation of t.  The loop is
 * launched as a CUDA graph.  n_done receives the number of steps taken;
 * ms_total (nullable) the device time of the loop measured with CUDA events
 * on the context stream; ms_kernel (nullable, forces per-launch events
 * instead of a graph) the summed durations of the step kernels alone. */
int lymph_run_steps(lymph_ctx* ctx, double stop_time, int64_t max_steps, double* t_inout,
                    int64_t* n_done, float* ms_total, float* ms_kernel);

/* Device-to-device copy between two state slots. */
int lymph_copy_state(lymph_ctx* ctx, int dst_slot, int src_slot);

/* Copies a state slot to / from host memory in the given layout
 * (synchronous on return).  LYMPH_LAYOUT_FORTRAN is transposed on the device
 * (a staging buffer of the state's size is allocated on the first such call),
 * so both layouts move as one direct copy; a page-locked host buffer moves
 * by DMA. */
int lymph_get_state(lymph_ctx* ctx, int slot, double* host, int layout);
int lymph_set_state(lymph_ctx* ctx, int slot, const double* host, int layout);

/* Checkpoint / resume of the time loop (the reference parses RESTART and
 * BKPFILE, src/Poly_readfile.f90:109-110, 129-131, but does not implement
 * them).  _save writes u^{n-1}, u^n, the caller's time t and step count, and
 * what identifies the run (a hash of the mesh descriptor's arrays, degree,
 * precision, dt, alpha, theta) to path, through a temporary file renamed at
 * the end.  _load, on a context built from the same mesh and parameters and
 * set up (lymph_make_matrices, lymph_make_rhs), restores the two states and
 * returns t and the step count; a file written for another run is refused
 * (LYMPH_ERR_INVALID).  Stepping on from a loaded checkpoint gives the same
 * bits as the uninterrupted run. */
int lymph_checkpoint_save(lymph_ctx* ctx, const char* path, double t, int64_t steps);
int lymph_checkpoint_load(lymph_ctx* ctx, const char* path, double* t, int64_t* steps);

/* COMPUTE_ERROR_L2_MATRIX_FREE (src/matrix_free.f90:1388-1418): sum over
 * polyhedra and components of du^T M_modal du, du = slot_uh - slot_uex.
 * Returns the sum of squares; the caller takes the square root, as the
 * driver does after its MPI_REDUCE (src/Lymph3D.f90:496-514). */
int lymph_error_l2(lymph_ctx* ctx, int slot_uh, int slot_uex, double* sumsq);

/* COMPUTE_ERROR_DG_MATRIX_FREE (src/matrix_free.f90:1421-1504): sum over
 * polyhedra of du_P^T (A_PP du_P + sum_Q A_PQ du_Q).  Assembles the A_dg
 * blocks into a temporary device buffer for the duration of the call. */
int lymph_error_dg(lymph_ctx* ctx, int slot_uh, int slot_uex, double* sumsq);

/* L2 error without any device allocation.  No counterpart in the reference:
 * it is the body of COMPUTE_ERROR_L2_MATRIX_FREE for callers that cannot
 * allocate device memory when they need the norm (a driver that gives all
 * device memory to its own pool, a process already at its device-memory cap,
 * a loop that must not take the synchronisation a cudaMalloc/cudaFree can
 * cause).  The caller passes device pointers to its own data:
 * d_mass_modal [n_poly][Np][Np] row-major (M_modal_loc), d_uh and d_uex
 * [n_poly][3Np]; the sum of squares is written to the host pointer sumsq.
 * The partial sums live in a static device array of 262,144 + 1 doubles
 * (2 MiB) that every GPU loading the library holds until the process exits;
 * n_poly above 262,144 is rejected with LYMPH_ERR_INVALID.  The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  With lazy module loading
 * (CUDA_MODULE_LOADING=LAZY, the CUDA default) that first call is also when
 * the 2 MiB are allocated on the device, so a caller that fills device
 * memory to a cap should make it before doing so.  The address is cached
 * per device ordinal for the life of the process: after a cudaDeviceReset
 * the cached address is stale, so do not call this again in that process.
 * Kernels run on the legacy default stream and the result is copied back
 * synchronously.  All calls share the one array: calls that overlap on the
 * GPU (from several host threads, or concurrently with other work on the
 * same device array) race. */
int lymph_error_l2_noalloc(const double* d_mass_modal, const double* d_uh, const double* d_uex, int32_t n_poly,
                           int32_t Np, double* sumsq);

/* ku = K u: the operator apply of TIME_STEP_MATRIX_FREE alone, before the
 * mass-matrix solve (the tp_KU mat-vecs over the self and neighbour blocks,
 * src/matrix_free.f90:1292-1338), in the context's precision: FP64 blocks,
 * FP32 blocks, or FP32 self blocks plus the matrix-free FP32 face terms
 * (LYMPH_MIXED_MF), rows summed in FP64.  u and ku are host arrays
 * [n_poly][3Np] (poly-major).  For parity checks of each precision's
 * operator; the step kernels fuse this apply with the rest of the step. */
int lymph_apply_operator(lymph_ctx* ctx, const double* u, double* ku);

/* Discrete energy of the leapfrog pair (u^a = slot_a, u^b = slot_b, one step
 * apart): E = 1/2 |(u^b - u^a)/dt|^2_M + 1/2 u^b . K u^a, the quantity the
 * scheme conserves without forcing when K is symmetric (SIPG, lambda = mu).
 * No counterpart in the reference; the learned surrogate's acceptance check. */
int lymph_energy(lymph_ctx* ctx, int slot_a, int slot_b, double* energy);

/* ---- learned surrogate network (no counterpart in the reference) -------
 * A per-polyhedron message-passing network, trained and evaluated by this
 * library's own CUDA kernels (BF16 weight copies, FP32 activations and
 * accumulation, FP32 Adam masters):
 *   h = relu(x W0 + b0);  L times: m = relu(h Wm + bm), a = W m,
 *   h += relu([h a g] Wu + bu);  y = h Wo + bo
 * W is a row-normalised face-area weight matrix (CSR), g the aggregated
 * shared-face geometry.  Parameters travel as one FP32 array in the order
 * W0 b0 (Wm bm Wu bu)xL Wo bo, matrices row-major [in x out]. */
typedef struct lymph_mpnn lymph_mpnn;
int lymph_mpnn_create(int32_t F, int32_t H, int32_t O, int32_t L, int32_t G, lymph_mpnn** out);
int lymph_mpnn_destroy(lymph_mpnn* net);
int64_t lymph_mpnn_num_params(const lymph_mpnn* net);
int lymph_mpnn_set_params(lymph_mpnn* net, const float* params);
int lymph_mpnn_get_params(lymph_mpnn* net, float* params, float* grads);
int lymph_mpnn_set_graph(lymph_mpnn* net, int32_t n_nodes, const int32_t* w_ptr, const int32_t* w_idx,
                         const float* w_val, const float* g);
int lymph_mpnn_forward(lymph_mpnn* net, const float* x, float* y);
int lymph_mpnn_loss_grad(lymph_mpnn* net, const float* x, const float* target, double* loss);
int lymph_mpnn_adam(lymph_mpnn* net, float lr, float beta1, float beta2, float eps);
int lymph_mpnn_launch_count(const lymph_mpnn* net, int64_t* count);
/* Average device time of `reps` inference forwards (no pre-activation
 * stores, as lymph_mpnn_forward runs it) on the features already on the
 * device (after a lymph_mpnn_forward), CUDA events on the network's stream. */
int lymph_mpnn_time_forward(lymph_mpnn* net, int32_t reps, double* ms);
/* 1 when the forward GEMMs run on the tensor cores (tcgen05, TF32 hi/lo split
 * of the activations, FP32 accumulation in tensor memory): H and O <= 256
 * and F, H, G multiples of 4; 0 when they run on the FP32 SIMT pipe (also
 * with LYMPH_MPNN_SIMT=1 in the environment at creation). */
int lymph_mpnn_uses_tensor_cores(const lymph_mpnn* net);
/* Gated output head: the O = 6 B network outputs per node are coefficients
 * alpha[j][b][i] and the effective output (2 nd columns, what forward
 * returns and the loss compares) is
 * yg[j][i*Np + m] = sum_b alpha[j][b][i] x[b*nd + i*Np + m], nd = 3 Np:
 * a per-node, per-component combination of the first B feature blocks. */
int lymph_mpnn_set_gate(lymph_mpnn* net, int32_t nd, int32_t B);

/* One surrogate block: with V0 = u^{n-1}, U0 = u^n, UN = u^{n+1} in the
 * context, predicts u^{n+1+k} for k = K-3, K-2, K-1 as the cubic Taylor
 * extrapolation u1 + k d1 + k(k+1)/2 d2 - k(k+1)(k+2)/6 a1
 * (d1 = u1 - u0, d2 = u1 - 2u0 + um, a1 = dt^2 M^-1 (K d1 - gdiff F_dyn),
 * one operator apply; gdiff = g(t_{n+1}) - g(t_n) of the source time
 * function) plus the network's correction sc_P (y3 phi3(k) + y4 phi4(k)) in
 * the Newton basis phi3 = k(k+1)(k+2)/K^3, phi4 = phi3 (k+3)/K, with
 * sc_P = (r4^2/r3) K^4/24 from the polyhedron's own scales r_b (RMS of u1,
 * d1, d2, a1 over its DOFs plus 1e-3 x the mesh-wide RMS); use_net = 0: the
 * extrapolation alone.  The features, normalised per polyhedron,
 * [u1/r1, d1/r2, d2/r3, a1/r4, log10 r2/r1, log10 r3/r2, log10 r4/r3,
 * lambda, mu, rho] are built on the device: F >= 4 * 3Np + 6;
 * the network's effective output is [y3 | y4] (2 * 3Np per polyhedron).
 * Afterwards V0 and UEX hold u^n, u^{n+1} (for a fallback), U0 and UN the
 * predicted u^{n+K-2}, u^{n+K-1}, and the network object the predicted
 * u^{n+K}.  K >= 4.  scales (nullable) receives the mesh-wide RMS s1..s4. */
int lymph_surrogate_predict(lymph_ctx* ctx, lymph_mpnn* net, int32_t K, int32_t use_net, double gdiff,
                            double* scales);

/* The feature rows lymph_surrogate_predict would build from the same
 * context state, copied to x (host, n_poly x F floats); scales (nullable, 4
 * doubles) receives s1..s4, a1 (nullable, n_poly x 3Np doubles) the
 * operator term, sig (nullable, n_poly x 4 doubles) the per-polyhedron
 * scales r1..r4.  For training samples from solver runs. */
int lymph_surrogate_features(lymph_ctx* ctx, lymph_mpnn* net, double gdiff, float* x, double* scales, double* a1,
                             double* sig);

/* The blocks of the surrogate block's operator apply (a1): on = 1 uses an
 * FP32 copy of an FP64 context's blocks (made on first use; faster, a1 then
 * carries FP32 rounding, ~1e-5 relative), on = 0 (default) the context's own. */
int lymph_surrogate_apply_fp32(lymph_ctx* ctx, int32_t on);

/* After one plain step from the predicted pair (U0 = u^{n+K-1}, UN = the
 * stepped u^{n+K}): residual = |UN - predicted u^{n+K}| / |UN|. */
int lymph_surrogate_residual(lymph_ctx* ctx, lymph_mpnn* net, double* residual);

/* Judge of a block on the device.  phase 0 keeps the pair (U0, UN) in the
 * network's scratch; phase 1, after the block was redone plainly, returns
 * rel = |(U0, UN) - kept| / |(U0, UN)|.  Phase 1 must precede the next
 * lymph_surrogate_predict (they share the scratch). */
int lymph_surrogate_judge(lymph_ctx* ctx, lymph_mpnn* net, int32_t phase, double* rel);

/* Nodal values of the field in `slot` at the four vertices of every
 * tetrahedron, out (host) [n_tet][4][3]: the reference's u_nod_vet(DIM, 4,
 * num_elem_loc) in the same memory order.  Replaces the evaluation loop of
 * EXPORT_SOLUTION (solution_processing.f90:62-194); the VTK / VTU / PVD
 * writers of export_file_formats.f90 are host code (export.py). */
int lymph_nodal_values(lymph_ctx* ctx, int slot, double* out);

/* Aliases with the names the project specification uses for the two error
 * routines (COMPUTE_ERROR_L2_FREE / COMPUTE_ERROR_DG_FREE). */
int lymph_compute_error_l2_free(lymph_ctx* ctx, int slot_uh, int slot_uex, double* sumsq);
int lymph_compute_error_dg_free(lymph_ctx* ctx, int slot_uh, int slot_uex, double* sumsq);

/* Debug / parity access to the assembled data (a3 of the reference path).
 * lymph_get_pattern: row_ptr[n_poly+1], col[n_blocks] (neighbour polyhedron
 * of each block; the self block comes first in each row).
 * lymph_get_blocks: vals[n_blocks][3Np][3Np] row-major (row = test dof of the
 * row polyhedron, column = trial dof of the column polyhedron), FP64 even in
 * mixed precision (the FP32 values are widened). */
int lymph_get_pattern(lymph_ctx* ctx, int32_t* row_ptr, int32_t* col);
int lymph_get_blocks(lymph_ctx* ctx, int which, double* vals);
/* The self blocks the step kernels apply, vals[n_poly][3Np][3Np] row-major:
 * the FP64 blocks, or the stored FP32 values widened (the mixed precisions:
 * the tensor-core assembly of MAKE_STIFFNESS_VOLUME + MAKE_STIFFNESS_FACE's
 * self terms, src/assemble_element.f90:24-77, 404-661).  A read-back for
 * parity checks; no counterpart in the reference. */
int lymph_get_self_blocks(lymph_ctx* ctx, double* vals);
/* Mass data per polyhedron, [n_poly][Np][Np] row-major: which = 0 M_loc (rho
 * weighted), 1 M_modal_loc, 2 R_M_loc (upper Cholesky factor), 3 R_M_modal_loc,
 * 4 the inverse of M_loc the step kernel applies. */
int lymph_get_mass(lymph_ctx* ctx, int which, double* vals);
/* RHS vectors [n_poly][3Np] (which = LYMPH_RHS_STAT / LYMPH_RHS_DYN). */
int lymph_get_rhs(lymph_ctx* ctx, int which, double* vals);
/* Per-polyhedron bounding box [n_poly][6] (xmin,xmax,ymin,ymax,zmin,zmax)
 * and diameter hk [n_poly] (CREATE_BBOX_EL). */
int lymph_get_poly_geometry(lymph_ctx* ctx, double* bbox, double* hk);

/* Point source for the rhs selected by `which`: rhs[P] = dir_i phi_m(x0) for
 * the polyhedron P of tetrahedron `tet` (find it with lymph_mesh_find_tet),
 * zero elsewhere; its time dependence (e.g. a Ricker wavelet) comes through
 * the time-function values of lymph_batch_run.  No counterpart in the
 * reference's path (its only source is the double couple of
 * src/matrix_free.f90:602-664, modelled on FIND_ELEM_FROM_POINT,
 * src/find_tet.f90:82-124, for the point lookup). */
int lymph_make_rhs_point(lymph_ctx* ctx, int which, int32_t tet, const double* x0, const double* dir);

/* Double-couple seismic source, the loop over PolyData%val_sism_el of
 * MAKE_RHS_FREE (matrix_free.f90:602-664) with MAKE_DOUBLE_COUPLE
 * (assemble_element.f90:116-167) and moment_density
 * (problem_data_and_properties.f90:317-335): ADDS to RHS `which`
 * (LYMPH_RHS_STAT / _DYN) the load int_T M : grad(phi) over tetrahedron
 * `tet` (find it with lymph_mesh_find_tet), M = (s n^T + n s^T) M0 / |T|,
 * s the strike vector, n the fault normal.  Each call takes its own s, n
 * and M0 (the reference reads the first source's for every source,
 * matrix_free.f90:647-652).  Call after MAKE_RHS_FREE, which zeroes the
 * vector; the reference adds the couple before the forcing terms, so the
 * source polyhedron's entries differ from it by rounding. */
int lymph_make_rhs_double_couple(lymph_ctx* ctx, int which, int32_t tet, const double* s, const double* n, double M0);

/* Time step after creation (e.g. from a CFL bound). */
int lymph_set_dt(lymph_ctx* ctx, double dt);
int lymph_get_dt(const lymph_ctx* ctx, double* dt);

/* Largest eigenvalue modulus of M^-1 K by `iters` power iterations on the
 * device operator; the leapfrog scheme is stable for dt < 2/sqrt(lam).
 * Replaces the placeholder COMPUTE_CFL (src/checks.f90:14-39), which only
 * tests dt against hmax. */
int lymph_max_eigenvalue(lymph_ctx* ctx, int32_t iters, double* lam);

/* The triangle rule of the LYMPH_MIXED_MF neighbour terms for degree p
 * (1..4): *n nodes; if xyw is not null it receives (xi, eta, w) per node on
 * the reference triangle (0,0), (1,0), (0,1), weights summing to 1/2.  Exact
 * to degree 2p, the degree of the face integrands, like the reference's
 * collapsed Gauss rule (mapping_quadrature_2D, Poly_ref_mappings.f90:137-186),
 * with fewer nodes.  Needs no device. */
int lymph_mf_face_rule(int32_t p, int32_t* n, double* xyw);

/* ---- many problems in one persistent launch per step -------------------
 * No counterpart in the reference (one problem per MPI job).  A batch
 * references n assembled contexts (same precision; any degrees, meshes and
 * dt).  lymph_batch_run advances every problem n_steps leapfrog steps
 * (TIME_STEP_MATRIX_FREE each) with one persistent kernel per step over all
 * (problem, polyhedron) items (LYMPH_MIXED_MF: one per degree present, each
 * over that degree's items), launched as CUDA graphs; gvals holds the
 * time-function value of every problem at every step, [n][n_steps].  Results
 * equal stepping each context alone, bit for bit, with the default schedule
 * (see lymph_batch_autotune for tuned tile shapes). */
typedef struct lymph_batch lymph_batch;
int lymph_batch_create(lymph_ctx* const* ctxs, int32_t n, lymph_batch** out);
int lymph_batch_destroy(lymph_batch* batch);
int lymph_batch_run(lymph_batch* batch, int64_t n_steps, const double* gvals, float* ms_total);
/* Times trial_steps steps for each candidate (1..4 persistent CTAs per SM,
 * for LYMPH_MIXED_MF 1..what one SM holds of the lowest degree's kernel, each
 * degree's grid capped at what the SMs hold of its own kernel; items
 * largest-cost-first or problem-major; for
 * LYMPH_FP64 / LYMPH_MIXED also three tile shapes, the column slices per
 * degree) and keeps the fastest; the problems' states are restored
 * afterwards.  The choice is cached per batch signature in $LYMPH_TUNE_CACHE
 * (default ~/.cache/lymph3d_gb300_tune2.txt) and reused when use_cache is
 * non-zero.  With tile shape 0 (the default before tuning) results equal
 * stepping each context alone bit for bit; the other shapes group each
 * row's partial sums differently: deterministic, equal up to rounding. */
int lymph_batch_autotune(lymph_batch* batch, int32_t trial_steps, int32_t use_cache, int32_t* grid, int32_t* order);
/* The current schedule: grid size, item order, tile shape (any pointer may be null). */
int lymph_batch_schedule(const lymph_batch* batch, int32_t* grid, int32_t* order, int32_t* shape);
int lymph_batch_launch_count(const lymph_batch* batch, int64_t* count);

/* Number of kernels this context launched so far (all kinds). */
int lymph_launch_count(const lymph_ctx* ctx, int64_t* count);

/* Device bytes the context holds (operator blocks, state, geometry). */
int lymph_device_bytes(const lymph_ctx* ctx, int64_t* bytes);

/* Measured FP64 FMA throughput of the current device, TFLOP/s (independent
 * FMA chains in registers, CUDA events): the roofline denominator of the
 * FP64 step kernel, which the FP64 pipe bounds.  No reference counterpart. */
int lymph_fp64_peak(int32_t iters, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* LYMPH3D_GPU_H */
