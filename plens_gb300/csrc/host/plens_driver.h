// plens_driver.h -- host driver with the public call chain of the reference's class PLENS
// (dgsem/plens.h:898-910; used by main.cc:96-106): declare_parameters, read_mesh, set_NS,
// set_dof_handler, set_sol_vecs, set_IC, set_BC, set_blender, read_time_settings, run.
// The hot path runs on the GPU through include/plens_gpu.h.
#pragma once

#include <memory>
#include <string>

#include "plens_gpu.h"
#include "prm.h"
#include "setup.h"

namespace plens {

class PLENS {
public:
    // Parses `prm_file` (input.prm in the working directory for the command-line driver).
    PLENS(int mapping_degree, int fe_degree, const std::string& prm_file = "input.prm");
    ~PLENS();
    void declare_parameters();
    void read_mesh();
    void set_NS();
    void set_dof_handler();
    void set_sol_vecs();
    void set_IC();
    void set_BC();
    void set_blender();
    void read_time_settings();
    // while (cur_time < end_time) update(); writing the state (.vtu, .pvd, .times, restart .ar)
    // every `write frequency` steps and at the end, and the final state to
    // <directory>/<base file name>.state (raw FP64 [5][ndof]).
    void run();

private:
    void build_if_needed();
    ParameterHandler prm_;
    int mhod_, degree_;
    std::string base_dir_;
    std::unique_ptr<Case> case_;
    plens_ctx* ctx_ = nullptr;
};

}  // namespace plens
