// capi.cpp -- extern "C" surface of the host setup chain (include/plens_host.h).
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "plens_host.h"
#include "output.h"
#include "setup.h"

struct plens_case {
    std::unique_ptr<plens::Case> c;
};

namespace {
thread_local std::string g_last_error;
}

extern "C" {

int plens_case_create(const char* prm_text, const char* base_dir, int mapping_degree,
                      int fe_degree, plens_case** out)
{
    return plens_case_create_ex(prm_text, base_dir, mapping_degree, fe_degree, nullptr, out);
}

int plens_case_create_ex(const char* prm_text, const char* base_dir, int mapping_degree,
                         int fe_degree, plens_geometry_fn geometry, plens_case** out)
{
    if (out) *out = nullptr;
    if (!prm_text || !out) {
        g_last_error = "null argument";
        return 1;
    }
    try {
        plens::ParameterHandler prm;
        plens::declare_parameters(prm);
        prm.parse_input_from_string(prm_text);
        auto* h = new plens_case();
        h->c = plens::build_case(prm, mapping_degree, fe_degree, base_dir ? base_dir : "", geometry);
        *out = h;
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

const char* plens_case_last_error(void) { return g_last_error.c_str(); }
void plens_case_destroy(plens_case* c) { delete c; }
const plens_mesh_desc* plens_case_mesh(const plens_case* c) { return &c->c->mesh; }
const plens_params* plens_case_params(const plens_case* c) { return &c->c->params; }
plens_params* plens_case_params_mut(plens_case* c) { return &c->c->params; }
int64_t plens_case_n_cells(const plens_case* c) { return c->c->n_cells; }
int64_t plens_case_n_dofs(const plens_case* c) { return c->c->n_dofs; }

int plens_case_setup_times(const plens_case* c, double* seconds)
{
    if (!c || !seconds) return 1;
    for (int i = 0; i < 4; ++i) seconds[i] = c->c->setup_seconds[i];
    return 0;
}

int plens_case_initial_state(const plens_case* c, double* U)
{
    std::memcpy(U, c->c->U0.data(), sizeof(double) * c->c->U0.size());
    return 0;
}

int plens_write_vtu(const plens_case* c, const char* path, const double* U, const double* avars,
                    const double* alpha, const double* alpha_d, double loc_dt)
{
    if (!c || !path || !U) {
        g_last_error = "null argument";
        return 1;
    }
    try {
        plens::Snapshot s;
        s.U = U;
        s.avars = avars;
        s.alpha = alpha;
        s.alpha_d = alpha_d;
        s.loc_dt = loc_dt;
        plens::write_vtu(path, *c->c, s);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

int plens_write_pvd(const char* path, int64_t n, const double* times, const char* const* files)
{
    if (!path || n < 0 || (n > 0 && (!times || !files))) {
        g_last_error = "null argument";
        return 1;
    }
    try {
        std::vector<std::pair<double, std::string>> e;
        for (int64_t i = 0; i < n; ++i) e.emplace_back(times[i], files[i]);
        plens::write_pvd(path, e);
        return 0;
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return 1;
    }
}

int plens_write_archive(const plens_case* c, const char* path, const double* U, double time, int64_t n_steps,
                        int64_t output_counter)
{
    if (!c || !path || !U) {
        g_last_error = "null argument";
        return 1;
    }
    try {
        plens::write_archive(path, *c->c, U, time, n_steps, output_counter);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

int plens_read_archive(const plens_case* c, const char* path, double* U, double* time, int64_t* n_steps,
                       int64_t* output_counter)
{
    if (!c || !path || !U) {
        g_last_error = "null argument";
        return 1;
    }
    try {
        plens::read_archive(path, c->c->degree, c->c->n_cells, c->c->n_dofs, U, time, n_steps, output_counter);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

int plens_case_dof_xyz(const plens_case* c, double* xyz)
{
    std::memcpy(xyz, c->c->dof_xyz.data(), sizeof(double) * c->c->dof_xyz.size());
    return 0;
}

double plens_case_start_time(const plens_case* c) { return c->c->start_time; }
double plens_case_end_time(const plens_case* c) { return c->c->end_time; }

double plens_case_eval_expr(const plens_case* c, int32_t idx, double x, double y, double z, double t)
{
    return c->c->exprs.eval(idx, x, y, z, t);
}

const char* plens_case_prm_echo(const plens_case* c) { return c->c->prm_echo.c_str(); }

int plens_expr_eval_string(const char* src, double x, double y, double z, double t, double* out)
{
    try {
        plens::ExprTable tab;
        const int32_t i = tab.add(src);
        *out = tab.eval(i, x, y, z, t);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

int plens_gll_1d(int n_points, double* nodes, double* weights)
{
    try {
        std::vector<double> x, w;
        plens::gll_1d(n_points, x, w);
        std::memcpy(nodes, x.data(), sizeof(double) * x.size());
        std::memcpy(weights, w.data(), sizeof(double) * w.size());
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

}  // extern "C"
