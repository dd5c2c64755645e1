/*
 * plens_gpu.h -- C ABI of the GB300 (sm_103a) implementation of PLENS's per-RK-stage
 * right-hand side and time update.
 *
 * The reference has no plugin or FFI for this path: the path is the private method set of
 * class PLENS (dgsem/plens.h:827-896), i.e. calc_rhs() (dgsem/plens.cc:3688-3779),
 * calc_time_step() (dgsem/plens.cc:3810-3912), multiply_time_step_to_rhs()
 * (dgsem/plens.cc:3925-3940) and update()/update_rk4() (dgsem/plens.cc:4334-4518), working on
 * member PETSc vectors. Each entry point below names the reference routine it replaces.
 *
 * Conventions (the ABI is plain C: pointers, sizes, status codes; no exceptions cross it):
 *  - P = degree+1; a cell holds P^3 GLL nodes numbered lexicographically, x fastest
 *    (dgsem/cell_dof_info.h:60-88); the global dof index of node l of cell c is c*P^3 + l.
 *  - Conservative state vectors are structure-of-arrays [5][ndof] in the order
 *    (rho, rho u, rho v, rho w, rho E) (modelling/var_enums.h:25-41); auxiliary variables are
 *    [9][ndof] in the order (txx, txy, txz, tyy, tyz, tzz, qx, qy, qz) (modelling/avars.h:14).
 *  - Faces of a cell are numbered 0..5 = -x,+x,-y,+y,-z,+z of the reference cell; face-local
 *    dof numbering follows dgsem/face_dof_info.h:92-150.
 *  - Host pointers passed in are borrowed for the duration of the call and copied.
 *  - One host thread per context; all device work runs on the context's own stream; every
 *    call returns after its work completed unless its name ends in _async.
 */
#ifndef PLENS_GPU_H
#define PLENS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define PLENS_GPU_OK 0
#define PLENS_GPU_E_INVALID 1    /* bad argument or unsupported option (AssertThrow in the reference) */
#define PLENS_GPU_E_CUDA 2       /* a CUDA runtime call failed */
#define PLENS_GPU_E_POSITIVITY 3 /* rho<=0 or e<=0 at some dof (reference: std::exit, plens.cc:2531-2546) */
#define PLENS_GPU_E_TIMEOUT 4    /* a bounded device wait gave up */

/* ------------------------------------------------------------- flux scheme enums
 * Same order as NavierStokes::inv_surf_flux_scheme / inv_vol_flux_scheme
 * (modelling/navier_stokes.h:161-183). */
enum plens_inv_surf_flux {
    PLENS_ISF_HLLC = 0,
    PLENS_ISF_RUSANOV = 1,
    PLENS_ISF_AUSM_PLUS_UP = 2,
    PLENS_ISF_RUSANOV_HLLC = 3,
    PLENS_ISF_RUSANOV_AUSM_PLUS_UP = 4,
    PLENS_ISF_MODIFIED_SW = 5,
    PLENS_ISF_CHANDRASHEKHAR = 6,
    PLENS_ISF_KENNEDY_GRUBER = 7,
    PLENS_ISF_RUSANOV_KENNEDY_GRUBER = 8,
    PLENS_ISF_ISMAIL_ROE = 9
};
enum plens_inv_vol_flux {
    PLENS_IVF_CHANDRASHEKHAR = 0,
    PLENS_IVF_KENNEDY_GRUBER = 1,
    PLENS_IVF_ISMAIL_ROE = 2
};

/* ------------------------------------------------------------ boundary conditions
 * One descriptor per boundary id; the types are the BCs:: classes of IBCs/. */
enum plens_bc_type {
    PLENS_BC_NONE = 0,
    PLENS_BC_FREE = 1,              /* IBCs/free.cc:16-59 */
    PLENS_BC_OUTFLOW = 2,           /* IBCs/outflow.cc:18-75 */
    PLENS_BC_UNIFORM_INFLOW = 3,    /* IBCs/uniform_inflow.cc:23-77 */
    PLENS_BC_UNIFORM_TEMP_WALL = 4, /* IBCs/uniform_temp_wall.cc:17-104 */
    PLENS_BC_SYMMETRY = 5,          /* IBCs/symmetry.cc:17-98 */
    PLENS_BC_EMPTY = 6,             /* IBCs/empty.cc:15-91 */
    PLENS_BC_PERIODIC = 7,          /* IBCs/periodic.cc:18-165 */
    PLENS_BC_INSULATED_WALL = 8,    /* IBCs/insulated_wall.cc:17-102 */
    PLENS_BC_VARYING_INFLOW = 9,    /* IBCs/varying_inflow.cc:17-141 */
    PLENS_BC_ZPG_INFLOW = 10        /* IBCs/zpg_inflow.cc:9-55 */
};

typedef struct plens_bc_desc {
    int32_t type;       /* enum plens_bc_type */
    int32_t expr_p;     /* varying inflow: expression index of p(x,y,z,t), else -1 */
    int32_t expr_T;     /* varying inflow: expression index of T(x,y,z,t), else -1 */
    int32_t expr_vel[3];/* varying inflow: expression indices of the velocity components */
    double p;           /* prescribed p (outflow) */
    double T;           /* prescribed T (uniform temp wall) */
    double vel[3];      /* prescribed / wall velocity */
    double cons[5];     /* prescribed conservative state (uniform inflow) */
} plens_bc_desc;

/* ------------------------------------------------------------------ expressions
 * muparser-style expressions (deal.II FunctionParser in the reference) compiled on the host to
 * a stack bytecode that the device and host evaluate identically. Variables: x,y,z,t. */
typedef struct plens_expr_insn {
    int32_t op;   /* opcode, see plens_gb300/csrc/common/expr.h */
    int32_t arg;  /* variable index / arity / jump target */
    double val;   /* literal */
} plens_expr_insn;

/* ------------------------------------------------------------------- parameters */
/* FP64: every operation in FP64 (the reference's arithmetic).
 * MIXED: the flux differencing, surface fluxes, subcell residual, viscous terms, indicator, CFL
 *   estimate and network in FP32; the state, the three RK registers and their accumulation, the
 *   metric terms and Jacobians (stored and read in FP64; FP32 arithmetic uses their rounding), the
 *   1/det J scaling of the residual, the positivity decision and the conservative face fluxes'
 *   sums in FP64.
 * MIXED_R32: as MIXED, but the RK registers hold dt*R in FP32, combined in FP32, and the FP32
 *   arithmetic reads FP32 images of the metric terms (made once at creation), scaling the residual
 *   by 1/det J in FP32; only the final state update U + inc is FP64. Fewer bytes per DOF-stage. */
enum plens_precision { PLENS_PRECISION_FP64 = 0, PLENS_PRECISION_MIXED = 1, PLENS_PRECISION_MIXED_R32 = 2 };
enum plens_sensor { PLENS_SENSOR_MODAL = 0, PLENS_SENSOR_LEARNED = 1 };

typedef struct plens_params {
    int32_t degree;            /* N (fe degree) */
    /* gas model: NavierStokes (modelling/navier_stokes.h:141-507) */
    double gamma, R, Pr, mu0, T0, S;   /* R = R0/M */
    int32_t const_viscosity;   /* 1 reproduces the CONST_VISCOSITY build switch (mu = mu0) */
    int32_t inv_surf_flux;     /* enum plens_inv_surf_flux */
    int32_t inv_vol_flux;      /* enum plens_inv_vol_flux */
    int32_t plens_2d;          /* 1 reproduces the PLENS_2D switch (rho w RHS zeroed) */
    /* blender (dgsem/blender_calculator.cc, "blender parameters" subsection) */
    int32_t blender_variable;  /* 0 pxrho, 1 p, 2 rho */
    int32_t blender_function;  /* 0 Hennemann, 1 linear */
    double threshold_factor, threshold_exp_factor, sharpness_factor, alpha_min, alpha_max;
    int32_t expr_wall_blender_limit;   /* expression of t */
    int32_t expr_vis_blending_region;  /* expression of x,y,z,t at cell centres */
    int32_t expr_courant;              /* expression of t */
    int32_t do_filtering;              /* TV filter (blender_calculator.cc:196-259) */
    /* time integration */
    int32_t rk_order;          /* 4: RK4(3)5[3R+]N; 3: SSP-RK3 */
    /* local time stepping (calc_time_step, dgsem/plens.cc:3880-3911) */
    int32_t local_stepping;        /* "request local stepping" */
    int32_t limit_local_step;      /* "limit local time step" */
    double local_start_time;       /* per-cell steps only while t > this ("local stepping start time") */
    double local_nbr_factor;       /* dt_c <= factor * unlimited dt of each interior-face neighbour */
    double local_global_factor;    /* dt_c <= factor * global dt */
    /* error norms of the output steps (PLENS::write, dgsem/plens.cc:4234-4243) */
    int32_t calc_ss_error;         /* "calculate steady state error": rho E of each step start is kept */
    int32_t calc_conv_error;       /* "convergence/calculate error" (variable: density) */
    int32_t expr_conv_exact;       /* "convergence/exact solution": expression of x,y,z,t */
    /* precision / learned sensor (new; no counterpart in the reference) */
    int32_t precision;         /* enum plens_precision */
    int32_t sensor;            /* enum plens_sensor */
    int32_t judge_every;       /* learned sensor: recompute the modal blender every k-th step */
    double judge_alpha_tol;    /* learned sensor: per-cell alpha error that triggers fallback */
    /* boundary conditions, indexed by boundary id (0..n_bc-1) */
    int32_t n_bc;
    const plens_bc_desc* bcs;
    /* expression table */
    int32_t n_expr;
    const int32_t* expr_offset;  /* [n_expr] first instruction */
    const int32_t* expr_length;  /* [n_expr] instruction count */
    int32_t n_expr_insn;
    const plens_expr_insn* expr_code;
} plens_params;

/* ------------------------------------------------------------ mesh description
 * Everything the hot path needs from the reference's setup chain (read_mesh, set_dof_handler,
 * form_neighbor_face_matchings, calc_metric_terms: dgsem/plens.cc:699-1009, 1574-1682),
 * produced once on the host. */
typedef struct plens_mesh_desc {
    int32_t degree;
    int64_t n_cells;
    /* per-dof metric terms (dgsem/metric_terms.cc:67-142), SoA over ndof = n_cells*P^3 */
    const double* detJ;         /* [ndof] */
    const double* Ja;           /* [9][ndof]: Ja[(dir*3+comp)*ndof+dof] = (J a^dir)_comp */
    const double* Jinv;         /* [9][ndof]: Jinv[(r*3+c)*ndof+dof] = d xi_r / d x_c */
    /* per-cell data */
    const double* h_min;        /* [n_cells] minimum vertex distance */
    const double* cell_center;  /* [n_cells][3] vertex average */
    const int32_t* cell_nbr;    /* [n_cells][6] interior neighbour, -1 on any boundary (periodic too) */
    const int32_t* cell_face_bc;/* [n_cells][6] boundary id of boundary faces, -1 interior */
    /* face tasks: each interior face once (owner = lower cell index), each boundary face
     * (periodic included) once per side */
    int64_t n_face_tasks;
    const int32_t* ft_cell;      /* [n_face_tasks] */
    const int32_t* ft_face;      /* [n_face_tasks] 0..5 */
    const int32_t* ft_nbr_cell;  /* interior: neighbour; periodic: partner cell; else -1 */
    const int32_t* ft_nbr_face;  /* interior/periodic: neighbour/partner face; else -1 */
    const int32_t* ft_bc;        /* boundary id, -1 interior */
    const int32_t* ft_nbr_fdof;  /* [n_face_tasks][P^2] matching face-local dof on the other side */
    const double* ft_normal;     /* [n_face_tasks][P^2][3] unit outward normal of the owner side */
    const double* ft_xyz;        /* [n_face_tasks][P^2][3] face dof location */
    /* QGauss(N+1) quadrature of the error norms (VectorTools::integrate_difference); null when
     * no error norm is requested. Gauss points are numbered like the dofs (c*P^3 + i + P j + P^2 k). */
    const double* gauss_interp;  /* [P][P]: GLL Lagrange basis i at Gauss point q, at [q*P+i] */
    const double* q_wJ;          /* [ndof] quadrature weight x det J at the Gauss point */
    const double* q_xyz;         /* [3][ndof] Gauss point location (convergence error only) */
} plens_mesh_desc;

typedef struct plens_ctx plens_ctx;

/* ------------------------------------------------------------------ lifecycle */

/* Replaces the device-facing half of the setup chain (set_sol_vecs, calc_metric_terms, set_BC:
 * dgsem/plens.cc:1025-1097, 1646-1682, 1219-1440): uploads the mesh description, the parameters
 * and the BC descriptors, allocates all device buffers. */
int plens_gpu_create(const plens_mesh_desc* mesh, const plens_params* params, plens_ctx** out);
int plens_gpu_destroy(plens_ctx* ctx);
/* Message of the last failed call on this context (never NULL). With ctx = NULL: the message of
 * the last failed context-free call (plens_gpu_time_step_noalloc) on the calling thread. */
const char* plens_gpu_last_error(const plens_ctx* ctx);
/* Number of CUDA kernels this library launched on the context so far. */
int64_t plens_gpu_kernel_launches(const plens_ctx* ctx);
/* The cudaStream_t the context launches on (as an opaque pointer). */
void* plens_gpu_stream(const plens_ctx* ctx);

/* Kernel timing on the context stream: when enabled, CUDA events bracket every launch of the
 * per-cell volume kernel (the dominant kernel); plens_gpu_kernel_timing returns the summed
 * elapsed milliseconds and the launch count since the last reset. */
int plens_gpu_set_kernel_timing(plens_ctx* ctx, int enable);
int plens_gpu_kernel_timing(plens_ctx* ctx, double* volume_ms, int64_t* volume_launches);

/* ----------------------------------------------------------------- state I/O
 * Replaces the g_cvars / gcrk_cvars buffer copies of PLENS::update (dgsem/plens.cc:4487-4514).
 * A page-locked (pinned, mapped) host buffer is read or written by the GPU through its device
 * mapping in one pass; any other host buffer goes through cudaMemcpy. */
int plens_gpu_set_state(plens_ctx* ctx, const double* U /* [5][ndof] */);
int plens_gpu_get_state(plens_ctx* ctx, double* U /* [5][ndof] */);
/* Simulation clock kept on the device (PLENS::cur_time, PLENS::n_time_steps). */
int plens_gpu_set_time(plens_ctx* ctx, double t, int64_t n_steps);
int plens_gpu_get_time(plens_ctx* ctx, double* t, int64_t* n_steps, double* last_dt);

/* ----------------------------------------------------------------- hot path */

/* One right-hand-side evaluation at the current state and time: PLENS::calc_rhs
 * (dgsem/plens.cc:3688-3779) including assert_positivity, calc_aux_vars, calc_blender and
 * calc_surf_flux. R_out ([5][ndof], may be NULL) receives the residual before the time-step
 * multiplication. Returns PLENS_GPU_E_POSITIVITY if assert_positivity would have aborted. */
int plens_gpu_rhs(plens_ctx* ctx, double* R_out);

/* PLENS::calc_time_step (dgsem/plens.cc:3810-3912) at the current state and time, global time
 * stepping: dt = min over dofs of Co/(N^1.5 (max_k (Jinv^T u)_k + a/h + N^2 mu/(h^2 rho))). */
int plens_gpu_time_step(plens_ctx* ctx, double* dt_out);

/* Stable time step of a caller-owned state, allocating nothing. No counterpart in the reference:
 * it is for callers that may not allocate device memory -- a framework that owns all GPU memory
 * through its own pool and forbids libraries from calling cudaMalloc, or a loop that must not
 * allocate while it runs. Same result as plens_gpu_time_step of an FP64 context (a mixed-precision
 * context evaluates the step in FP32 and differs by about 1e-6 relative), but on device arrays
 * the caller passes: U [5][ndof], Jinv [9][ndof] and h_min [n_cells] in the layouts of plens_mesh_desc, the
 * gas of `params`, the Courant number `courant` (capped to 0.9 when >= 1), and dt_out, one
 * double in device memory that receives the step (before any end-time clip). Runs on `stream`
 * (a cudaStream_t, may be NULL) and returns without synchronising.
 * Scratch: the per-cell steps go to a library-owned device array of PLENS_GPU_NOALLOC_MAX_CELLS
 * doubles (2 MiB) that every GPU using the library keeps until the process exits; larger meshes
 * return PLENS_GPU_E_INVALID. All calls share that array: calls that overlap on the GPU race.
 * The first call on each device looks the array up (cudaGetSymbolAddress) and keeps its address
 * for the life of the process; make that first call before any stream capture, and do not call
 * this entry point after a cudaDeviceReset of that device (the kept address would be stale).
 * Errors: PLENS_GPU_E_INVALID for bad arguments or a mesh beyond the scratch array, and
 * PLENS_GPU_E_CUDA for a failed launch or a CUDA error already pending from earlier work (which
 * is reported, not cleared); plens_gpu_last_error(NULL) gives the message of the last failed
 * call on the calling thread. */
#define PLENS_GPU_NOALLOC_MAX_CELLS (1 << 18)
int plens_gpu_time_step_noalloc(const double* U, const double* Jinv, const double* h_min, int64_t n_cells,
                                int32_t degree, const plens_params* params, double courant, double* dt_out,
                                void* stream);

/* n_steps calls of PLENS::update (dgsem/plens.cc:4484-4518): each step computes dt on the device
 * at stage 1, clips it to end_time - t (dgsem/plens.cc:4341), runs the RK stages
 * (update_rk4 dgsem/plens.cc:4334-4403 or update_rk3 4420-4475) and advances the device clock.
 * Steps stop early once t >= end_time. The _async form returns without synchronising; errors
 * raised by the device (positivity, learned-sensor fallback counters) are reported by the next
 * synchronising call. */
int plens_gpu_advance(plens_ctx* ctx, int64_t n_steps, double end_time);
int plens_gpu_advance_async(plens_ctx* ctx, int64_t n_steps, double end_time);
int plens_gpu_synchronize(plens_ctx* ctx);

/* A sequence of independent states on this context's mesh and parameters (ensemble members,
 * the cases of a parameter study, restarts), each made the current state at time t0 with the step
 * counter at 0, advanced by n_steps steps as plens_gpu_advance advances it (stopping at end_time),
 * and handed back. The reference advances one state per run, `while (cur_time < end_time)
 * update();` (PLENS::run, dgsem/plens.cc:1509-1550); a host loop of plens_gpu_set_state,
 * plens_gpu_advance and plens_gpu_get_state does the same per member with the transfers in series.
 * Here the transfers run on two copy streams beside the steps: member j+1 is copied in and member
 * j-1 copied out while member j is advanced.
 *  - U_in[j], U_out[j]: host [5][ndof] buffers. Page-locked ones (cudaHostAlloc,
 *    cudaHostRegister) give the overlap; pageable ones give the same results in series.
 *    U_out[j] must not overlap any U_in[k], k > j.
 *  - t_out: NULL or count doubles, member j's clock after its steps.
 *  - Errors: the call returns the status of the first member that failed, named in
 *    plens_gpu_last_error (positivity: plens_gpu_first_bad_dof gives its dof); the outputs of
 *    the members before it are complete. With the learned sensor the call stops there (its
 *    fallback redoes failed steps from the host, so its members run one after the other);
 *    otherwise every member is advanced (each starts with a clear error state) and the later
 *    members' outputs are complete as well. No copy to or from the caller's buffers outlives
 *    the call. The context then holds the state and clock of the last member it advanced.
 *  - Device buffers for the two staged states and a page-locked status array are made on the
 *    first call (the array grows with count). */
int plens_gpu_advance_states(plens_ctx* ctx, int64_t count, const double* const* U_in, double* const* U_out,
                             double t0, int64_t n_steps, double end_time, double* t_out);

/* Error norms of the current state as PLENS::write logs them (dgsem/plens.cc:4234-4243), i.e.
 * at stage 1 of the next step, after its time step: the steady-state error
 * ||(rhoE - rhoE_old) / loc_dt|| / ||rhoE|| (calc_ss_error, 3985-4035; rhoE_old = rho E at the
 * start of the previous step, zero before the first) and the L2 error of density against the
 * exact-solution expression at the current time (calc_convergence_error, 4044-4098); L2 norms by
 * QGauss(N+1) quadrature. Either output may be NULL; asking for a norm that was not requested at
 * setup gives PLENS_GPU_E_INVALID. Synchronising. */
int plens_gpu_error_norms(plens_ctx* ctx, double* ss_error, double* conv_error);

/* The compacted troubled-cell list of the last RHS (mixed forms with the Chandrashekhar volume
 * flux at odd N, where the subcell residual runs over it): the cells with alpha > 0 in increasing
 * index order -- the cells calc_cell_lo_inv_residual (dgsem/plens.cc:3469-3583) runs on -- built
 * without atomics, so the same on every run. cells ([n_cells], may be NULL) receives the list,
 * *count its length. PLENS_GPU_E_INVALID for a context without a list. Synchronising. */
int plens_gpu_troubled_cells(plens_ctx* ctx, int32_t* cells, int64_t* count);

/* Per-cell scalars of the last RHS: PLENS::gcrk_alpha, gcrk_alpha_d, loc_time_steps. */
int plens_gpu_get_cell_scalars(plens_ctx* ctx, double* alpha, double* alpha_d, double* dt_cell);
/* Auxiliary variables of the last viscous RHS ([9][ndof]): PLENS::gcrk_avars. */
int plens_gpu_get_avars(plens_ctx* ctx, double* avars);
/* Learned sensor: evaluate the network's two hidden layers on the tensor cores (tcgen05, 3xTF32)
 * or on the CUDA cores (enable = 0). At degree 3 the tensor-core form is one fused kernel (the
 * features, both layers and the judge's plain indicator for handed-back cells) and the default,
 * measured faster; at other degrees it is a two-kernel form and the CUDA cores are the default.
 * No reference counterpart. */
int plens_gpu_set_sensor_tensor_cores(plens_ctx* ctx, int enable);
/* Modal indicator of a mixed-precision context of degree 3 (the blender's change of basis,
 * dgsem/blender_calculator.cc:123-177 with dgsem/change_of_basis_matrix.h:74-98): the 64 x 64
 * change of basis of 128 cells at a time on the tensor cores (tcgen05, 3xTF32) when enable != 0
 * -- the default, measured faster -- else the separable transform on the CUDA cores.
 * PLENS_GPU_E_INVALID for other contexts. */
int plens_gpu_set_indicator_tensor_cores(plens_ctx* ctx, int enable);
/* Compacted troubled-cell list of a mixed-precision context with the Chandrashekhar volume flux:
 * the subcell kernel finds the cell at each list position itself, from the smoothing kernel's
 * per-block counts and ballots (enable != 0; the default where the counts fit its shared memory,
 * up to 1,048,448 cells), or a list kernel writes the list first (enable = 0; the form of larger
 * meshes). Both give the same list and the same residual, bit for bit. PLENS_GPU_E_INVALID for
 * other contexts, or enable != 0 on a larger mesh. No reference counterpart. */
int plens_gpu_set_list_decoding(plens_ctx* ctx, int enable);
/* Asynchronous snapshot for data output (replaces the host reads of PLENS::write,
 * dgsem/plens.cc:4170-4322): _begin copies U, alpha, alpha_d, the auxiliary variables (viscous)
 * and the clock on the context's stream into a device buffer, then to library-owned pinned host
 * memory on a second stream, and returns at once -- steps launched after it overlap the copy.
 * _end waits for that copy and hands the snapshot out (any pointer may be NULL; avars [9][ndof]).
 * One snapshot may be pending at a time. */
int plens_gpu_snapshot_begin(plens_ctx* ctx);
int plens_gpu_snapshot_end(plens_ctx* ctx, double* U, double* alpha, double* alpha_d, double* avars,
                           double* time, int64_t* n_steps, double* dt);
/* First dof that failed the positivity check of the last failing call (-1 if none). */
int plens_gpu_first_bad_dof(const plens_ctx* ctx, int64_t* dof);
/* Self-test of the mixed form's integer-pipe FP64 <-> FP32 conversions (no reference
 * counterpart; test hook): n seeded samples (raw encodings, values in and around the float
 * range, rounding ties) converted both by them and by the hardware conversions on the device;
 * *mismatches receives the number of results whose encodings differ (NaN compared as NaN). */
int plens_gpu_selftest_conversions(int64_t n, uint64_t seed, int64_t* mismatches);

/* ----------------------------------------------------- learned troubled-cell sensor
 * New component (no counterpart in the reference): an MLP (64 -> 64 -> 64 -> 1, GELU,
 * sigmoid*alpha_max) that replaces the modal indicator BlenderCalculator::get_blender
 * (dgsem/blender_calculator.cc:123-177); the neighbour smoothing (dgsem/plens.cc:2926-2947) then
 * runs on its output and also emits the compacted troubled-cell list. Values below
 * max(alpha_min, 0.01) are set to 0. Weights are FP32, laid out W1[64][64], b1[64], W2[64][64],
 * b2[64], W3[64], b3[1] (row-major, out x in). */
#define PLENS_MLP_IN 64
#define PLENS_MLP_HIDDEN 64
#define PLENS_MLP_N_PARAMS (64 * 64 + 64 + 64 * 64 + 64 + 64 + 1)
int plens_gpu_set_sensor_weights(plens_ctx* ctx, const float* params /* [PLENS_MLP_N_PARAMS] */);
/* Learned-sensor statistics: steps judged; fallbacks = cells handed back to the plain modal
 * indicator, summed over the judged steps (a cell whose alpha error exceeds the judge tolerance
 * keeps the plain indicator until the next judged step; a step redone after a positivity
 * failure counts every cell); the max per-cell alpha error seen; and the number of cells the
 * subcell kernel ran on in the last RHS (the length of the compacted troubled-cell list). */
int plens_gpu_sensor_stats(plens_ctx* ctx, int64_t* judged, int64_t* fallbacks,
                           double* max_alpha_err, int64_t* lo_cells_last);
/* Training pairs of the current state: x [n_cells][64] FP32, the sensor input (nodal rho*p
 * interpolated to the 4^3 GLL nodes, divided by its mean, minus 1); y [n_cells] FP32, the modal
 * indicator's alpha before neighbour smoothing (with the wall override). */
int plens_gpu_sensor_pairs(plens_ctx* ctx, float* x, float* y);

/* MLP training on the device with the library's own forward, backward and Adam kernels.
 * x: [n][64] FP32 (host), y: [n] FP32 (host). params: [PLENS_MLP_N_PARAMS] in/out (host).
 * Mini-batch SGD with Adam(lr, beta1=0.9, beta2=0.999, eps=1e-8); the sample order of each
 * epoch is a permutation drawn from `seed`. loss_out[epochs] receives the mean-squared error
 * of each epoch (may be NULL). Standalone: needs no context. */
int plens_gpu_mlp_train(const float* x, const float* y, int64_t n, float* params,
                        int32_t epochs, int32_t batch, float lr, float alpha_max,
                        uint64_t seed, float* loss_out);
/* One forward+backward pass over a batch, for gradient checks: loss (mean squared error) and
 * the gradient of the loss with respect to every parameter. */
int plens_gpu_mlp_loss_grad(const float* x, const float* y, int64_t n, const float* params,
                            float alpha_max, float* loss, float* grad /* [PLENS_MLP_N_PARAMS] */);
/* Inference only: alpha for n samples. */
int plens_gpu_mlp_infer(const float* x, int64_t n, const float* params, float alpha_max,
                        float* alpha /* [n] */);

/* ------------------------------------------------------- geometry setup on the GPU
 * The two parts of the reference's setup chain whose cost grows with the mesh and the degree:
 *  - calc_metric_terms (dgsem/plens.cc:1646-1682) with MetricTerms<3>::reinit
 *    (dgsem/metric_terms.cc:67-142): location, J, det J, J^-1 and the contravariant vectors
 *    Ja^i = a_j x a_k (cyclic) at every node of a tensor rule, from the degree-m Lagrange
 *    interpolant of each cell's (m+1)^3 support points (MappingQGeneric(m));
 *  - form_neighbor_face_matchings (dgsem/plens.cc:1574-1627): for every face task and face dof
 *    the matching face dof of the other side, found by location (O(P^4) per face), with the
 *    unit outward normal of FEFaceValues::normal_vector (dgsem/plens.cc:1751-1756, 1797).
 * The support points (the manifold description), the neighbour/periodic topology and the face
 * task list stay on the host (plens_host.h). The arithmetic is the host setup's, operation for
 * operation and without multiply-add contraction, so both produce the same bits. */
typedef struct plens_geometry_job {
    /* mapping at the nodes of a tensor rule (the GLL nodes, or the Gauss points of the error
     * norms); node l of cell c is c*n_points^3 + l, l = i + n_points (j + n_points k) */
    int32_t n_points;         /* rule points per direction */
    int32_t n_support;        /* support points per direction, mapping degree + 1 */
    int64_t n_cells;
    const double* support;    /* [n_cells][n_support^3][3], point s = i + n_support (j + n_support k) */
    const double* basis;      /* [n_points][n_support]: 1D Lagrange basis of the support points */
    const double* dbasis;     /* [n_points][n_support]: its derivative */
    double* xyz;              /* out [3][n_nodes], or NULL */
    double* detJ;             /* out [n_nodes], or NULL */
    double* Ja;               /* out [9][n_nodes] as in plens_mesh_desc, or NULL */
    double* Jinv;             /* out [9][n_nodes] as in plens_mesh_desc, or NULL */
    int64_t first_bad_cell;   /* out: first cell with det J <= 0 at a node, or -1 */
    /* face dofs of the face tasks (n_face_tasks = 0: none). Needs the GLL rule of the degree
     * (n_points = degree + 1) with xyz and Ja requested. */
    int64_t n_face_tasks;
    const int32_t* ft_cell;      /* as in plens_mesh_desc */
    const int32_t* ft_face;
    const int32_t* ft_nbr_cell;  /* -1: no other side, the face dof matches itself */
    const int32_t* ft_nbr_face;
    const int32_t* ft_skip_dir;  /* periodic direction, left out of the match distance (the match
                                    must then keep the face-dof order), or -1 */
    const double* ft_tol;        /* match tolerance of the task (distance < tol) */
    int32_t* ft_nbr_fdof;        /* out [n_face_tasks][P^2] */
    double* ft_normal;           /* out [n_face_tasks][P^2][3] */
    double* ft_xyz;              /* out [n_face_tasks][P^2][3] */
    int64_t first_unmatched;     /* out: first task*P^2 + q without a matching face dof, or -1 */
    int64_t first_misoriented;   /* out: first periodic task*P^2 + q matched to another q, or -1 */
} plens_geometry_job;

/* Runs a geometry job on the current device: allocates its device buffers, computes, copies the
 * outputs to the job's host arrays and frees the buffers before returning. Returns
 * PLENS_GPU_E_INVALID for bad sizes or pointers (the first_* outputs are results, not errors). */
int plens_gpu_setup_geometry(plens_geometry_job* job);
typedef int (*plens_geometry_fn)(plens_geometry_job* job);

#ifdef __cplusplus
}
#endif

#endif /* PLENS_GPU_H */
