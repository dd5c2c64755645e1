/*
 * plens_host.h -- C ABI of the host-side setup chain: builds, from the reference's input.prm
 * format, the mesh description, parameters and initial state that plens_gpu.h consumes.
 *
 * Replaces the reference's setup chain PLENS::PLENS / declare_parameters / read_mesh / set_NS /
 * set_dof_handler / set_sol_vecs / set_IC / set_BC / set_blender / read_time_settings
 * (dgsem/plens.cc:13-1499, main.cc:96-106). Host only: loads and runs without a GPU.
 */
#ifndef PLENS_HOST_H
#define PLENS_HOST_H

#include <stdint.h>

#include "plens_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plens_case plens_case;

/* Parses prm text (input.prm contents), builds mesh, metric terms, face tables, BCs and the
 * initial condition. base_dir resolves relative file names (mesh, IC file). Returns 0 or 1; on
 * failure *out is NULL and plens_case_last_error() holds the message. */
int plens_case_create(const char* prm_text, const char* base_dir, int mapping_degree,
                      int fe_degree, plens_case** out);
/* As plens_case_create, with the function that runs the geometry jobs (metric terms and face-dof
 * matching) when the prm entry "GB300/geometry setup" is "gpu": normally plens_gpu_setup_geometry
 * of the GPU library, passed in so that this library needs no GPU. With "host" (the default)
 * or a NULL function the host computes them. */
int plens_case_create_ex(const char* prm_text, const char* base_dir, int mapping_degree,
                         int fe_degree, plens_geometry_fn geometry, plens_case** out);
const char* plens_case_last_error(void);
void plens_case_destroy(plens_case* c);

const plens_mesh_desc* plens_case_mesh(const plens_case* c);
const plens_params* plens_case_params(const plens_case* c);
/* Mutable parameters (precision / sensor switches may be flipped before plens_gpu_create). */
plens_params* plens_case_params_mut(plens_case* c);
int64_t plens_case_n_cells(const plens_case* c);
int64_t plens_case_n_dofs(const plens_case* c);
/* Wall seconds of the setup phases: [0] mesh and parameters, [1] geometry (support points,
 * metric terms, face dofs, error-norm quadrature), [2] topology, BCs and face-task list,
 * [3] initial condition. */
int plens_case_setup_times(const plens_case* c, double* seconds /* [4] */);
/* Initial state [5][ndof] (PLENS::set_IC) and dof locations [3][ndof]. */
int plens_case_initial_state(const plens_case* c, double* U);
int plens_case_dof_xyz(const plens_case* c, double* xyz);
double plens_case_start_time(const plens_case* c);
double plens_case_end_time(const plens_case* c);
/* Evaluates expression `idx` of the case's expression table. */
double plens_case_eval_expr(const plens_case* c, int32_t idx, double x, double y, double z, double t);
/* All parameters with their values (ParameterHandler::print_parameters); valid until destroy. */
const char* plens_case_prm_echo(const plens_case* c);

/* Data output of PLENS::write (dgsem/plens.cc:4170-4322) with post_process (3950-3963): a VTK XML
 * unstructured grid of the case's mesh (each cell's GLL nodes as points, N^3 linear sub-hexahedra)
 * with txx..qz (if avars is not NULL), rho, p, T, u, v, w as point data and subdomain, alpha,
 * alpha_d, loc_dt, global_active_cell_index as cell data. U: [5][ndof]; avars: [9][ndof] or NULL;
 * alpha, alpha_d: [n_cells] or NULL. Returns 0, or 1 with plens_case_last_error set. */
int plens_write_vtu(const plens_case* c, const char* path, const double* U, const double* avars,
                    const double* alpha, const double* alpha_d, double loc_dt);
/* ParaView collection record (DataOutBase::write_pvd_record) of n (time, file) pairs. */
int plens_write_pvd(const char* path, int64_t n, const double* times, const char* const* files);
/* Restart archive of the state (replaces the SolutionTransfer archives that the reference's
 * "from archive restart" initial condition reads, IBCs/from_archive_restart.cc:23-73): this
 * build's own format -- a header (magic, degree, cells, dofs, steps, output counter, time) and
 * U [5][ndof] in FP64. The "from archive restart" IC type of input.prm reads it back. */
int plens_write_archive(const plens_case* c, const char* path, const double* U, double time, int64_t n_steps,
                        int64_t output_counter);
int plens_read_archive(const plens_case* c, const char* path, double* U, double* time, int64_t* n_steps,
                       int64_t* output_counter);

/* Stand-alone helpers for the known-answer tests. */
int plens_expr_eval_string(const char* src, double x, double y, double z, double t, double* out);
int plens_gll_1d(int n_points, double* nodes, double* weights);

#ifdef __cplusplus
}
#endif

#endif /* PLENS_HOST_H */
