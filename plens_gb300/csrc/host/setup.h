// setup.h -- host-side producer of everything the hot path consumes: the reference's setup chain
// (PLENS::read_mesh, set_NS, set_dof_handler, form_neighbor_face_matchings, calc_metric_terms,
// set_sol_vecs, set_IC, set_BC, set_blender, read_time_settings: dgsem/plens.cc:699-1499,
// 1574-1682) restated without deal.II. The result is a Case: a plens_mesh_desc, a plens_params
// and the initial state, all owned by the Case.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "expr_compile.h"
#include "plens_gpu.h"
#include "prm.h"

namespace plens {

// ------------------------------------------------------------------------- 1D operators
// Gauss-Lobatto-Legendre nodes and weights on [0,1] (deal.II QGaussLobatto<1>, the reference cell
// is [0,1]^3: dgsem/plens.h "vol_contrib" note 1).
void gll_1d(int n_points, std::vector<double>& nodes, std::vector<double>& weights);
// Gauss-Legendre nodes and weights on [0,1] (deal.II QGauss<1>).
void gauss_1d(int n_points, std::vector<double>& nodes, std::vector<double>& weights);
// Lagrange basis through `nodes` evaluated / differentiated at x.
double lagrange(const std::vector<double>& nodes, int j, double x);
double lagrange_deriv(const std::vector<double>& nodes, int j, double x);

// ----------------------------------------------------------------------------- meshes
// Hexahedral mesh with deal.II's lexicographic vertex numbering (v = i + 2j + 4k) and face
// numbering (0..5 = -x,+x,-y,+y,-z,+z).
struct HexMesh {
    std::vector<std::array<double, 3>> vertices;
    std::vector<std::array<int64_t, 8>> cells;
    std::vector<std::array<int32_t, 6>> face_bid;  // boundary id of boundary faces, -1 otherwise
    // manifold: 0 = straight (Q1), 1 = cylinder around axis (axis_dir, axis_point), 2 = nose
    // cylinder: cells whose centre lies beyond the plane through axis_point normal to axis_dir are
    // spherical about nose_center, the others cylindrical about the axis through axis_point
    int manifold = 0;
    std::array<double, 3> axis_dir{{0, 0, 1}}, axis_point{{0, 0, 0}}, nose_center{{0, 0, 0}};
};

struct BoxSpec {
    std::array<double, 3> lo{{0, 0, 0}}, hi{{1, 1, 1}};
    std::array<int, 3> n{{1, 1, 1}};
    std::array<int32_t, 6> bid{{1, 2, 3, 4, 5, 6}};
    // optional split of the -y face at x = split_x: faces with centre x > split_x get split_bid
    bool split = false;
    double split_x = 0;
    int32_t split_bid = 0;
};
HexMesh make_box(const BoxSpec& spec);

struct OMeshSpec {
    double r_inner = 1, r_outer = 10;
    int n_radial = 16, n_azimuthal = 16, n_z = 1;
    double first_cell = 1e-3;  // height of the first radial cell (geometric clustering)
    double z_length = 0.1;
    int32_t bid_inner = 1, bid_outer_front = 2, bid_outer_back = 3, bid_zlo = 4, bid_zhi = 5;
};
HexMesh make_o_mesh(const OMeshSpec& spec);

// gmsh ASCII 2.2 reader (hexahedra + physical quad boundary tags), replacing GridIn::read_msh.
HexMesh read_msh(const std::string& filename);

// ------------------------------------------------------------------------------ case
struct Case {
    int degree = 1, mapping_degree = 1;
    int64_t n_cells = 0, n_dofs = 0;
    // mesh description arrays
    std::vector<double> detJ, Ja, Jinv, h_min, cell_center, dof_xyz;  // dof_xyz: [3][ndof]
    std::vector<int32_t> cell_nbr, cell_face_bc;
    std::vector<int32_t> ft_cell, ft_face, ft_nbr_cell, ft_nbr_face, ft_bc, ft_nbr_fdof;
    std::vector<double> ft_normal, ft_xyz;
    // quadrature of the error norms (empty unless requested)
    std::vector<double> gauss_interp, q_wJ, q_xyz;
    // parameters
    std::vector<plens_bc_desc> bcs;
    ExprTable exprs;
    plens_params params{};
    plens_mesh_desc mesh{};
    // time settings (PLENS::read_time_settings, dgsem/plens.cc:1473-1499)
    double start_time = 0, end_time = 1;
    int64_t starting_output_counter = 0, write_freq = 100;
    std::string output_dir = "result", base_file_name = "output";
    std::string sensor_weights_file;
    // initial state [5][ndof]
    std::vector<double> U0;
    std::string prm_echo;
    // wall seconds of the setup phases: mesh and parameters, geometry (support points, metric
    // terms, face dofs, error-norm quadrature), topology/BCs/face-task list, initial condition
    double setup_seconds[4] = {0, 0, 0, 0};

    void finalize_pointers();  // points params/mesh at the owned vectors
};

// Declares every entry the driver understands (PLENS::declare_parameters,
// dgsem/plens.cc:73-650, plus the "GB300" and "mesh/builtin" subsections of this build).
void declare_parameters(ParameterHandler& prm);

// Builds a Case from parsed parameters. `base_dir` resolves relative file names (mesh, IC).
// `geometry` runs the metric-term and face-dof jobs when "GB300/geometry setup" is "gpu"
// (plens_gpu_setup_geometry of the GPU library); with "host" they run here.
std::unique_ptr<Case> build_case(const ParameterHandler& prm, int mapping_degree, int fe_degree,
                                 const std::string& base_dir, plens_geometry_fn geometry = nullptr);

// Conservative state from primitives (NavierStokes::prim_to_cons, navier_stokes.h:366-379).
void prim_to_cons(double gamma, double rho, const double vel[3], double p, double cons[5]);

}  // namespace plens
