// output.h -- data output of the driver: PLENS::write / post_process (dgsem/plens.cc:4170-4322,
// 3950-3963) restated without deal.II's DataOut, and a native restart archive replacing the
// SolutionTransfer archives read by the "from archive restart" initial condition
// (IBCs/from_archive_restart.cc:23-73).
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "setup.h"

namespace plens {

// Fields of one snapshot; any pointer but U may be null.
struct Snapshot {
    const double* U = nullptr;        // [5][ndof]
    const double* avars = nullptr;    // [9][ndof] (viscous runs)
    const double* alpha = nullptr;    // [n_cells]
    const double* alpha_d = nullptr;  // [n_cells]
    double loc_dt = 0;                // the step size in use (global time stepping)
};

// VTK XML unstructured grid (.vtu, binary inline, UInt64 headers): each cell's (N+1)^3 GLL nodes
// as points, its N^3 sub-hexahedra as linear cells (deal.II's DataOut without higher-order cells
// writes the same patches). Point data: txx..qz (viscous), rho, p, T, u, v, w (post_process: p and
// T from the NavierStokes relations); cell data: subdomain, alpha, alpha_d, loc_dt,
// global_active_cell_index.
void write_vtu(const std::string& path, const Case& c, const Snapshot& s);

// ParaView collection record of (time, file) pairs (DataOutBase::write_pvd_record).
void write_pvd(const std::string& path, const std::vector<std::pair<double, std::string>>& entries);

// Restart archive: a header (magic, degree, cells, dofs, time, steps, output counter) and the
// conservative state [5][ndof] in FP64.
void write_archive(const std::string& path, const Case& c, const double* U, double time, int64_t n_steps,
                   int64_t output_counter);
// Reads an archive written for the same mesh and degree; throws on any mismatch.
void read_archive(const std::string& path, int degree, int64_t n_cells, int64_t n_dofs, double* U, double* time,
                  int64_t* n_steps, int64_t* output_counter);

}  // namespace plens
