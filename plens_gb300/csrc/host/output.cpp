// output.cpp -- see output.h.
#include "output.h"

#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace plens {

namespace {

const char kB64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

void base64(std::ostream& os, const unsigned char* p, size_t n)
{
    size_t i = 0;
    for (; i + 3 <= n; i += 3) {
        const unsigned v = (unsigned)p[i] << 16 | (unsigned)p[i + 1] << 8 | p[i + 2];
        os << kB64[v >> 18] << kB64[(v >> 12) & 63] << kB64[(v >> 6) & 63] << kB64[v & 63];
    }
    if (n - i == 1) {
        const unsigned v = (unsigned)p[i] << 16;
        os << kB64[v >> 18] << kB64[(v >> 12) & 63] << "==";
    } else if (n - i == 2) {
        const unsigned v = (unsigned)p[i] << 16 | (unsigned)p[i + 1] << 8;
        os << kB64[v >> 18] << kB64[(v >> 12) & 63] << kB64[(v >> 6) & 63] << '=';
    }
}

// one binary inline data array: a base64 UInt64 byte count, then the base64 data (VTK encodes
// the two separately)
template <class T>
void data_array(std::ostream& os, const char* type, const std::string& name, int ncomp, const std::vector<T>& v)
{
    os << "        <DataArray type=\"" << type << "\"";
    if (!name.empty()) os << " Name=\"" << name << "\"";
    if (ncomp > 1) os << " NumberOfComponents=\"" << ncomp << "\"";
    os << " format=\"binary\">\n";
    const uint64_t nbytes = sizeof(T) * v.size();
    base64(os, reinterpret_cast<const unsigned char*>(&nbytes), sizeof(nbytes));
    base64(os, reinterpret_cast<const unsigned char*>(v.data()), nbytes);
    os << "\n        </DataArray>\n";
}

}  // namespace

void write_vtu(const std::string& path, const Case& c, const Snapshot& s)
{
    if (!s.U) throw std::runtime_error("write_vtu: no state");
    const int P = c.degree + 1, N = c.degree, P2 = P * P, P3 = P2 * P;
    const int64_t nc = c.n_cells, nd = c.n_dofs, nsub = nc * (int64_t)N * N * N;
    const double gamma = c.params.gamma, cv = c.params.R / (c.params.gamma - 1);
    const double* U = s.U;

    std::vector<double> pts(3 * nd);
    for (int64_t i = 0; i < nd; ++i)
        for (int d = 0; d < 3; ++d) pts[3 * i + d] = c.dof_xyz[d * nd + i];
    // post_process (dgsem/plens.cc:3950-3963): p = NavierStokes::get_p, T = get_e / c_v, velocity
    std::vector<double> rho(nd), p(nd), T(nd), vel[3] = {std::vector<double>(nd), std::vector<double>(nd), std::vector<double>(nd)};
    for (int64_t i = 0; i < nd; ++i) {
        const double r = U[i], m[3] = {U[nd + i], U[2 * nd + i], U[3 * nd + i]}, E = U[4 * nd + i];
        double ske = m[0] * m[0];
        ske += m[1] * m[1];
        ske += m[2] * m[2];
        rho[i] = r;
        p[i] = (gamma - 1) * (E - 0.5 * ske / r);
        const double e = (E - 0.5 * ske / r) / r;
        T[i] = e / cv;
        for (int d = 0; d < 3; ++d) vel[d][i] = m[d] / r;
    }
    // N^3 linear sub-hexahedra per cell over its GLL nodes (VTK_HEXAHEDRON vertex order)
    std::vector<int64_t> conn(8 * nsub), offs(nsub);
    std::vector<uint8_t> types(nsub, 12);
    std::vector<float> sub(nsub, 0.0f), al(nsub, 0.0f), ald(nsub, 0.0f), ldt(nsub, (float)s.loc_dt), gidx(nsub);
    int64_t k = 0;
    for (int64_t cell = 0; cell < nc; ++cell)
        for (int kz = 0; kz < N; ++kz)
            for (int jy = 0; jy < N; ++jy)
                for (int ix = 0; ix < N; ++ix) {
                    const int64_t b = cell * P3;
                    auto node = [&](int i, int j, int l) { return b + (ix + i) + P * (jy + j) + P2 * (kz + l); };
                    const int64_t v[8] = {node(0, 0, 0), node(1, 0, 0), node(1, 1, 0), node(0, 1, 0),
                                          node(0, 0, 1), node(1, 0, 1), node(1, 1, 1), node(0, 1, 1)};
                    for (int q = 0; q < 8; ++q) conn[8 * k + q] = v[q];
                    offs[k] = 8 * (k + 1);
                    if (s.alpha) al[k] = (float)s.alpha[cell];
                    if (s.alpha_d) ald[k] = (float)s.alpha_d[cell];
                    gidx[k] = (float)cell;
                    ++k;
                }

    std::ofstream os(path, std::ios::binary);
    if (!os.good()) throw std::runtime_error("cannot open " + path);
    os << "<?xml version=\"1.0\"?>\n"
       << "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
       << "  <UnstructuredGrid>\n"
       << "    <Piece NumberOfPoints=\"" << nd << "\" NumberOfCells=\"" << nsub << "\">\n"
       << "      <PointData Scalars=\"rho\">\n";
    if (s.avars) {
        static const char* names[9] = {"txx", "txy", "txz", "tyy", "tyz", "tzz", "qx", "qy", "qz"};  // var_enums.h:39-41
        for (int m = 0; m < 9; ++m) data_array(os, "Float64", names[m], 1, std::vector<double>(s.avars + m * nd, s.avars + (m + 1) * nd));
    }
    data_array(os, "Float64", "rho", 1, rho);
    data_array(os, "Float64", "p", 1, p);
    data_array(os, "Float64", "T", 1, T);
    data_array(os, "Float64", "u", 1, vel[0]);
    data_array(os, "Float64", "v", 1, vel[1]);
    data_array(os, "Float64", "w", 1, vel[2]);
    os << "      </PointData>\n      <CellData>\n";
    data_array(os, "Float32", "subdomain", 1, sub);
    data_array(os, "Float32", "alpha", 1, al);
    data_array(os, "Float32", "alpha_d", 1, ald);
    data_array(os, "Float32", "loc_dt", 1, ldt);
    data_array(os, "Float32", "global_active_cell_index", 1, gidx);
    os << "      </CellData>\n      <Points>\n";
    data_array(os, "Float64", "", 3, pts);
    os << "      </Points>\n      <Cells>\n";
    data_array(os, "Int64", "connectivity", 1, conn);
    data_array(os, "Int64", "offsets", 1, offs);
    data_array(os, "UInt8", "types", 1, types);
    os << "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
    if (!os.good()) throw std::runtime_error("write failed: " + path);
}

void write_pvd(const std::string& path, const std::vector<std::pair<double, std::string>>& entries)
{
    std::ofstream os(path);
    if (!os.good()) throw std::runtime_error("Unable to open pvd file. Make sure the specified output directory exists.");
    os << "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
       << "  <Collection>\n";
    os.precision(17);
    for (const auto& e : entries)
        os << "    <DataSet timestep=\"" << e.first << "\" group=\"\" part=\"0\" file=\"" << e.second << "\"/>\n";
    os << "  </Collection>\n</VTKFile>\n";
}

namespace {
const char kMagic[8] = {'P', 'L', 'E', 'N', 'S', 'A', 'R', '1'};
struct ArchiveHeader {
    char magic[8];
    int64_t degree, n_cells, n_dofs, n_steps, output_counter;
    double time;
};
}  // namespace

void write_archive(const std::string& path, const Case& c, const double* U, double time, int64_t n_steps,
                   int64_t output_counter)
{
    ArchiveHeader h{};
    std::memcpy(h.magic, kMagic, 8);
    h.degree = c.degree;
    h.n_cells = c.n_cells;
    h.n_dofs = c.n_dofs;
    h.n_steps = n_steps;
    h.output_counter = output_counter;
    h.time = time;
    std::ofstream os(path, std::ios::binary);
    if (!os.good()) throw std::runtime_error("cannot open " + path);
    os.write(reinterpret_cast<const char*>(&h), sizeof(h));
    os.write(reinterpret_cast<const char*>(U), sizeof(double) * 5 * c.n_dofs);
    if (!os.good()) throw std::runtime_error("write failed: " + path);
}

void read_archive(const std::string& path, int degree, int64_t n_cells, int64_t n_dofs, double* U, double* time,
                  int64_t* n_steps, int64_t* output_counter)
{
    std::ifstream is(path, std::ios::binary);
    if (!is.good()) throw std::runtime_error("cannot open archive " + path);
    ArchiveHeader h{};
    is.read(reinterpret_cast<char*>(&h), sizeof(h));
    if (!is || std::memcmp(h.magic, kMagic, 8) != 0) throw std::runtime_error("not a restart archive: " + path);
    if (h.degree != degree || h.n_cells != n_cells || h.n_dofs != n_dofs)
        throw std::runtime_error("archive " + path + " was written for another mesh or degree");
    is.read(reinterpret_cast<char*>(U), sizeof(double) * 5 * n_dofs);
    if (!is) throw std::runtime_error("archive " + path + " is truncated");
    if (time) *time = h.time;
    if (n_steps) *n_steps = h.n_steps;
    if (output_counter) *output_counter = h.output_counter;
}

}  // namespace plens
