// plens_driver.cpp -- see plens_driver.h.
#include "plens_driver.h"

#include "output.h"

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
    if (!case_) case_ = build_case(prm_, mhod_, degree_, base_dir_, &plens_gpu_setup_geometry);
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

namespace {
std::string counter_name(const std::string& base, int64_t counter)
{
    char buf[32];
    std::snprintf(buf, sizeof(buf), "_%06lld", (long long)counter);
    return base + buf;
}
}  // namespace

// PLENS::run + write (dgsem/plens.cc:1509-1550, 4170-4322): the state is written at every
// `write frequency`-th step and at the end -- a .vtu file per output (one process: no .pvtu), the
// .pvd collection, the .times log (counter, time, wall time), the .ss_error / .conv_error logs
// when those norms are requested, and a restart archive (.ar, read
// back by the "from archive restart" initial condition). Each output is an asynchronous device
// snapshot: the next `write frequency` steps are already running on the GPU while the host
// writes the files of the previous output.
void PLENS::run()
{
    set_sol_vecs();
    const std::string dir = case_->output_dir;
    mkdir(dir.c_str(), 0755);
    {
        std::ofstream f(dir + "/simulation_parameters.prm");
        f << case_->prm_echo << "\n# FE degree " << degree_ << "\n# Mapping degree " << case_->mapping_degree
          << "\n# Processors 1 (GPU)\n# DoFs per variable " << case_->n_dofs << "\n# Indicator: Hennemenn"
          << "\n# Lifting: entropy variables\n";
    }
    const std::string base = case_->base_file_name;
    std::ofstream times(dir + "/" + base + ".times", std::ios::app);
    // the error logs of write() (dgsem/plens.cc:4291-4319): counter, time, error
    const bool want_ss = case_->params.calc_ss_error != 0, want_conv = case_->params.calc_conv_error != 0;
    std::ofstream ss_log, conv_log;
    if (want_ss) ss_log.open(dir + "/" + base + ".ss_error", std::ios::app);
    if (want_conv) conv_log.open(dir + "/" + base + ".conv_error", std::ios::app);
    double ss_err = 0, conv_err = 0;
    // the norms of the state about to be snapshot (write() computes them at stage 1 of the step)
    auto error_norms = [&]() {
        if (want_ss || want_conv)
            check(plens_gpu_error_norms(ctx_, want_ss ? &ss_err : nullptr, want_conv ? &conv_err : nullptr), ctx_,
                  "error_norms");
    };
    const auto t0 = std::chrono::steady_clock::now();
    auto wall = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    const bool viscous = !(case_->params.mu0 < 1e-16);
    const bool learned = case_->params.sensor == PLENS_SENSOR_LEARNED;
    const int64_t nd = case_->n_dofs, nc = case_->n_cells;
    std::vector<double> U(5 * nd), alpha(nc), alpha_d(nc), avars(viscous ? 9 * nd : 0);
    std::vector<std::pair<double, std::string>> pvd;
    int64_t counter = case_->starting_output_counter;

    auto write_snapshot = [&]() {
        double t = 0, dt = 0;
        int64_t n = 0;
        check(plens_gpu_snapshot_end(ctx_, U.data(), alpha.data(), alpha_d.data(), viscous ? avars.data() : nullptr,
                                     &t, &n, &dt),
              ctx_, "snapshot_end");
        const std::string name = counter_name(base, counter);
        Snapshot s;
        s.U = U.data();
        s.avars = viscous ? avars.data() : nullptr;
        s.alpha = alpha.data();
        s.alpha_d = alpha_d.data();
        s.loc_dt = dt;
        write_vtu(dir + "/" + name + ".vtu", *case_, s);
        pvd.emplace_back(t, name + ".vtu");
        write_pvd(dir + "/" + base + ".pvd", pvd);
        write_archive(dir + "/" + name + ".ar", *case_, U.data(), t, n, counter);
        times << counter << " " << t << " " << wall() << "\n";
        times.flush();
        if (want_ss) ss_log << counter << " " << t << " " << ss_err << "\n" << std::flush;
        if (want_conv) conv_log << counter << " " << t << " " << conv_err << "\n" << std::flush;
        ++counter;
    };

    double t = case_->start_time, dt = 0;
    int64_t n = 0;
    check(plens_gpu_get_time(ctx_, &t, &n, &dt), ctx_, "get_time");
    error_norms();
    check(plens_gpu_snapshot_begin(ctx_), ctx_, "snapshot_begin");
    while (t < case_->end_time) {
        if (learned) {
            // the learned sensor's positivity fallback redoes steps from the host
            write_snapshot();
            check(plens_gpu_advance(ctx_, case_->write_freq, case_->end_time), ctx_, "advance");
        } else {
            check(plens_gpu_advance_async(ctx_, case_->write_freq, case_->end_time), ctx_, "advance_async");
            write_snapshot();  // overlaps the steps just launched
            check(plens_gpu_synchronize(ctx_), ctx_, "advance");
        }
        check(plens_gpu_get_time(ctx_, &t, &n, &dt), ctx_, "get_time");
        std::printf("Current time: %.9g, dt: %.6g, time steps: %lld, elapsed wall time: %.3f\n", t, dt, (long long)n,
                    wall());
        error_norms();
        check(plens_gpu_snapshot_begin(ctx_), ctx_, "snapshot_begin");
    }
    write_snapshot();
    check(plens_gpu_get_state(ctx_, U.data()), ctx_, "get_state");
    std::ofstream out(dir + "/" + base + ".state", std::ios::binary);
    out.write(reinterpret_cast<const char*>(U.data()), sizeof(double) * U.size());
}

}  // namespace plens
