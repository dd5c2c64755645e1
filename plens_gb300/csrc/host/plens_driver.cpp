// plens_driver.cpp -- see plens_driver.h.
#include "plens_driver.h"

#include <chrono>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <sys/stat.h>

namespace plens {

namespace {
void check(int rc, plens_ctx* c, const char* what)
{
    if (rc != PLENS_GPU_OK)
        throw std::runtime_error(std::string(what) + ": " + plens_gpu_last_error(c) + " (status " + std::to_string(rc) + ")");
}
}  // namespace

PLENS::PLENS(int mapping_degree, int fe_degree, const std::string& prm_file) : mhod_(mapping_degree), degree_(fe_degree)
{
    if (mapping_degree < 1) throw std::runtime_error("High order mapping degree must be >= 1.");
    declare_parameters();
    prm_.parse_input(prm_file);
    const size_t slash = prm_file.find_last_of('/');
    base_dir_ = (slash == std::string::npos) ? "." : prm_file.substr(0, slash);
}

PLENS::~PLENS()
{
    if (ctx_) plens_gpu_destroy(ctx_);
}

void PLENS::declare_parameters() { plens::declare_parameters(prm_); }

// The setup chain is built in one pass (mesh, NS model, dof tables, metric terms, BCs, IC and
// time settings depend on each other only through the Case); each step of the reference's chain
// triggers it if it has not run yet.
void PLENS::build_if_needed()
{
    if (!case_) case_ = build_case(prm_, mhod_, degree_, base_dir_);
}
void PLENS::read_mesh() { build_if_needed(); }
void PLENS::set_NS() { build_if_needed(); }
void PLENS::set_dof_handler() { build_if_needed(); }
void PLENS::set_sol_vecs()
{
    build_if_needed();
    if (!ctx_) check(plens_gpu_create(&case_->mesh, &case_->params, &ctx_), ctx_, "plens_gpu_create");
}
void PLENS::set_IC()
{
    set_sol_vecs();
    check(plens_gpu_set_state(ctx_, case_->U0.data()), ctx_, "set_state");
    check(plens_gpu_set_time(ctx_, case_->start_time, 0), ctx_, "set_time");
}
void PLENS::set_BC() { build_if_needed(); }
void PLENS::set_blender()
{
    build_if_needed();
    if (case_->params.sensor == PLENS_SENSOR_LEARNED) {
        std::ifstream f(case_->sensor_weights_file, std::ios::binary);
        if (!f.good()) throw std::runtime_error("cannot read sensor weights file " + case_->sensor_weights_file);
        std::vector<float> w(PLENS_MLP_N_PARAMS);
        f.read(reinterpret_cast<char*>(w.data()), sizeof(float) * w.size());
        if (!f) throw std::runtime_error("sensor weights file too short");
        set_sol_vecs();
        check(plens_gpu_set_sensor_weights(ctx_, w.data()), ctx_, "set_sensor_weights");
    }
}
void PLENS::read_time_settings() { build_if_needed(); }

void PLENS::run()
{
    set_sol_vecs();
    const std::string dir = case_->output_dir;
    mkdir(dir.c_str(), 0755);
    {
        std::ofstream f(dir + "/simulation_parameters.prm");
        f << case_->prm_echo << "\n# FE degree " << degree_ << "\n# Mapping degree " << case_->mapping_degree
          << "\n# Processors 1 (GPU)\n# DoFs per variable " << case_->n_dofs << "\n";
    }
    std::ofstream times(dir + "/" + case_->base_file_name + ".times");
    const auto t0 = std::chrono::steady_clock::now();
    double t = case_->start_time, dt = 0;
    int64_t n = 0;
    check(plens_gpu_get_time(ctx_, &t, &n, &dt), ctx_, "get_time");
    while (t < case_->end_time) {
        check(plens_gpu_advance(ctx_, case_->write_freq, case_->end_time), ctx_, "advance");
        check(plens_gpu_get_time(ctx_, &t, &n, &dt), ctx_, "get_time");
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("Current time: %.9g, dt: %.6g, time steps: %lld, elapsed wall time: %.3f\n", t, dt, (long long)n, wall);
        times << n << " " << t << " " << wall << "\n";
    }
    std::vector<double> U(5 * case_->n_dofs);
    check(plens_gpu_get_state(ctx_, U.data()), ctx_, "get_state");
    std::ofstream out(dir + "/" + case_->base_file_name + ".state", std::ios::binary);
    out.write(reinterpret_cast<const char*>(U.data()), sizeof(double) * U.size());
}

}  // namespace plens
