// setup.cpp -- see setup.h. Each block names the reference routine it restates.
#include "setup.h"
#include "output.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <fstream>
#include <map>
#include <random>
#include <sstream>
#include <stdexcept>

namespace plens {

// =================================================================================== 1D

void gll_1d(int n, std::vector<double>& nodes, std::vector<double>& weights)
{
    // Newton iteration for the roots of (1-x^2) P'_{n-1} on [-1,1], in long double, then mapped
    // to [0,1]; weights 2/(N(N+1) P_N(x)^2) halved.
    if (n < 2) throw std::runtime_error("GLL rule needs at least 2 points");
    const int N = n - 1;
    std::vector<long double> x(n), xold(n), P(static_cast<size_t>(n) * n);
    for (int i = 0; i < n; ++i) x[i] = std::cos(M_PI * static_cast<long double>(i) / N);
    for (int it = 0; it < 100; ++it) {
        long double diff = 0;
        for (int i = 0; i < n; ++i) {
            xold[i] = x[i];
            long double p0 = 1, p1 = x[i];
            long double pkm1 = p0, pk = p1;
            for (int k = 2; k <= N; ++k) {
                const long double pn = ((2 * k - 1) * x[i] * pk - (k - 1) * pkm1) / k;
                pkm1 = pk;
                pk = pn;
            }
            // pk = P_N, pkm1 = P_{N-1}
            if (N == 1) { pkm1 = p0; pk = p1; }
            x[i] = xold[i] - (x[i] * pk - pkm1) / (n * pk);
            diff = std::max(diff, std::fabs(x[i] - xold[i]));
            P[i] = pk;
        }
        if (diff < 1e-19L) break;
    }
    nodes.assign(n, 0);
    weights.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        long double pk, pkm1 = 1, pc = x[i];
        pk = pc;
        for (int k = 2; k <= N; ++k) {
            const long double pn = ((2 * k - 1) * x[i] * pk - (k - 1) * pkm1) / k;
            pkm1 = pk;
            pk = pn;
        }
        if (N == 1) pk = x[i];
        const long double w = 2.0L / (N * n * pk * pk);
        // ascending order on [0,1]
        nodes[n - 1 - i] = static_cast<double>((x[i] + 1) / 2);
        weights[n - 1 - i] = static_cast<double>(w / 2);
    }
    nodes[0] = 0.0;
    nodes[n - 1] = 1.0;
    for (int i = 0; i < n / 2; ++i) {  // exact symmetry about 1/2
        const double a = 0.5 * (nodes[i] + (1.0 - nodes[n - 1 - i]));
        nodes[i] = a;
        nodes[n - 1 - i] = 1.0 - a;
        const double w = 0.5 * (weights[i] + weights[n - 1 - i]);
        weights[i] = weights[n - 1 - i] = w;
    }
    if (n % 2 == 1) nodes[n / 2] = 0.5;
}

void gauss_1d(int n, std::vector<double>& nodes, std::vector<double>& weights)
{
    nodes.assign(n, 0);
    weights.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        long double x = std::cos(M_PI * (i + 0.75L) / (n + 0.5L)), dp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1, p1 = x;
            for (int k = 2; k <= n; ++k) {
                const long double pn = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = pn;
            }
            if (n == 1) { p1 = x; p0 = 1; }
            dp = n * (x * p1 - p0) / (x * x - 1);
            const long double dx = p1 / dp;
            x -= dx;
            if (std::fabs(dx) < 1e-20L) break;
        }
        nodes[n - 1 - i] = static_cast<double>((x + 1) / 2);
        weights[n - 1 - i] = static_cast<double>(1.0L / ((1 - x * x) * dp * dp));
    }
}

double lagrange(const std::vector<double>& nodes, int j, double x)
{
    double v = 1.0;
    for (size_t m = 0; m < nodes.size(); ++m)
        if (static_cast<int>(m) != j) v *= (x - nodes[m]) / (nodes[j] - nodes[m]);
    return v;
}

double lagrange_deriv(const std::vector<double>& nodes, int j, double x)
{
    double sum = 0.0;
    for (size_t k = 0; k < nodes.size(); ++k) {
        if (static_cast<int>(k) == j) continue;
        double term = 1.0 / (nodes[j] - nodes[k]);
        for (size_t m = 0; m < nodes.size(); ++m)
            if (static_cast<int>(m) != j && m != k) term *= (x - nodes[m]) / (nodes[j] - nodes[m]);
        sum += term;
    }
    return sum;
}

// ================================================================================ meshes

namespace {
// deal.II face -> cell-local vertex ids (GeometryInfo<3>::face_to_cell_vertices, standard
// orientation)
const int kFaceVerts[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5},
                              {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};

std::array<double, 3> face_center(const HexMesh& m, int64_t c, int f)
{
    std::array<double, 3> s{{0, 0, 0}};
    for (int v = 0; v < 4; ++v)
        for (int d = 0; d < 3; ++d) s[d] += 0.25 * m.vertices[m.cells[c][kFaceVerts[f][v]]][d];
    return s;
}
}  // namespace

HexMesh make_box(const BoxSpec& s)
{
    HexMesh m;
    const int nx = s.n[0], ny = s.n[1], nz = s.n[2];
    if (nx < 1 || ny < 1 || nz < 1) throw std::runtime_error("box subdivisions must be >= 1");
    auto vid = [&](int i, int j, int k) { return static_cast<int64_t>(i) + (nx + 1) * (j + static_cast<int64_t>(ny + 1) * k); };
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i)
                m.vertices.push_back({s.lo[0] + (s.hi[0] - s.lo[0]) * i / nx,
                                      s.lo[1] + (s.hi[1] - s.lo[1]) * j / ny,
                                      s.lo[2] + (s.hi[2] - s.lo[2]) * k / nz});
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                std::array<int64_t, 8> c;
                for (int v = 0; v < 8; ++v)
                    c[v] = vid(i + (v & 1), j + ((v >> 1) & 1), k + ((v >> 2) & 1));
                m.cells.push_back(c);
                std::array<int32_t, 6> fb{{-1, -1, -1, -1, -1, -1}};
                if (i == 0) fb[0] = s.bid[0];
                if (i == nx - 1) fb[1] = s.bid[1];
                if (j == 0) fb[2] = s.bid[2];
                if (j == ny - 1) fb[3] = s.bid[3];
                if (k == 0) fb[4] = s.bid[4];
                if (k == nz - 1) fb[5] = s.bid[5];
                m.face_bid.push_back(fb);
            }
    if (s.split) {
        for (size_t c = 0; c < m.cells.size(); ++c)
            if (m.face_bid[c][2] >= 0 && face_center(m, static_cast<int64_t>(c), 2)[0] > s.split_x)
                m.face_bid[c][2] = s.split_bid;
    }
    return m;
}

HexMesh make_o_mesh(const OMeshSpec& s)
{
    HexMesh m;
    const int nr = s.n_radial, nt = s.n_azimuthal, nz = s.n_z;
    if (nr < 1 || nt < 3 || nz < 1) throw std::runtime_error("bad o-mesh subdivisions");
    // geometric clustering: h1 (q^nr - 1)/(q - 1) = L
    const double L = s.r_outer - s.r_inner;
    double q = 1.0;
    if (s.first_cell * nr < L) {
        double lo = 1.0 + 1e-12, hi = 2.0;
        auto len = [&](double qq) { return s.first_cell * (std::pow(qq, nr) - 1) / (qq - 1); };
        while (len(hi) < L) hi *= 2;
        for (int it = 0; it < 200; ++it) {
            const double mid = 0.5 * (lo + hi);
            (len(mid) < L ? lo : hi) = mid;
        }
        q = 0.5 * (lo + hi);
    }
    std::vector<double> r(nr + 1);
    r[0] = s.r_inner;
    double h = (q == 1.0) ? L / nr : s.first_cell;
    for (int i = 1; i <= nr; ++i) {
        r[i] = r[i - 1] + h;
        h *= q;
    }
    r[nr] = s.r_outer;
    auto vid = [&](int i, int j, int k) {
        return static_cast<int64_t>(i) + (nr + 1) * ((j % nt) + static_cast<int64_t>(nt) * k);
    };
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j < nt; ++j)
            for (int i = 0; i <= nr; ++i) {
                const double th = 2.0 * M_PI * j / nt;
                m.vertices.push_back({r[i] * std::cos(th), r[i] * std::sin(th), s.z_length * k / nz});
            }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < nt; ++j)
            for (int i = 0; i < nr; ++i) {
                std::array<int64_t, 8> c;
                for (int v = 0; v < 8; ++v)
                    c[v] = vid(i + (v & 1), j + ((v >> 1) & 1), k + ((v >> 2) & 1));
                m.cells.push_back(c);
                std::array<int32_t, 6> fb{{-1, -1, -1, -1, -1, -1}};
                if (i == 0) fb[0] = s.bid_inner;
                if (i == nr - 1) fb[1] = s.bid_outer_front;  // resolved below by x of the face centre
                if (k == 0) fb[4] = s.bid_zlo;
                if (k == nz - 1) fb[5] = s.bid_zhi;
                m.face_bid.push_back(fb);
            }
    for (size_t c = 0; c < m.cells.size(); ++c)
        if (m.face_bid[c][1] >= 0)
            m.face_bid[c][1] = (face_center(m, static_cast<int64_t>(c), 1)[0] < 0) ? s.bid_outer_front
                                                                                    : s.bid_outer_back;
    m.manifold = 1;
    return m;
}

HexMesh read_msh(const std::string& filename)
{
    std::ifstream f(filename);
    if (!f.good()) throw std::runtime_error("Unable to open mesh file " + filename);
    HexMesh m;
    std::string tok;
    std::map<int64_t, int64_t> node_index;
    std::vector<std::pair<std::array<int64_t, 4>, int32_t>> quads;
    while (f >> tok) {
        if (tok == "$MeshFormat") {
            double ver;
            int ft, ds;
            f >> ver >> ft >> ds;
            if (ver >= 3.0 || ft != 0) throw std::runtime_error("only ASCII msh 2.x meshes are supported");
        } else if (tok == "$Nodes") {
            int64_t n;
            f >> n;
            for (int64_t i = 0; i < n; ++i) {
                int64_t id;
                double x, y, z;
                f >> id >> x >> y >> z;
                node_index[id] = static_cast<int64_t>(m.vertices.size());
                m.vertices.push_back({x, y, z});
            }
        } else if (tok == "$Elements") {
            int64_t n;
            f >> n;
            for (int64_t e = 0; e < n; ++e) {
                int64_t id;
                int type, ntags;
                f >> id >> type >> ntags;
                std::vector<int64_t> tags(ntags);
                for (auto& t : tags) f >> t;
                const int nn = (type == 5) ? 8 : (type == 3) ? 4 : (type == 15) ? 1 : (type == 1) ? 2 : (type == 2) ? 3 : -1;
                if (nn < 0) throw std::runtime_error("unsupported msh element type " + std::to_string(type));
                std::vector<int64_t> nodes(nn);
                for (auto& v : nodes) f >> v;
                if (type == 5) {
                    // gmsh hex (0,0,0)(1,0,0)(1,1,0)(0,1,0)(0,0,1)(1,0,1)(1,1,1)(0,1,1) ->
                    // deal.II lexicographic order
                    static const int perm[8] = {0, 1, 3, 2, 4, 5, 7, 6};
                    std::array<int64_t, 8> c;
                    for (int v = 0; v < 8; ++v) c[v] = node_index.at(nodes[perm[v]]);
                    m.cells.push_back(c);
                    m.face_bid.push_back({{-1, -1, -1, -1, -1, -1}});
                } else if (type == 3) {
                    std::array<int64_t, 4> q;
                    for (int v = 0; v < 4; ++v) q[v] = node_index.at(nodes[v]);
                    std::sort(q.begin(), q.end());
                    quads.emplace_back(q, ntags > 0 ? static_cast<int32_t>(tags[0]) : 0);
                }
            }
        }
    }
    std::map<std::array<int64_t, 4>, int32_t> qmap(quads.begin(), quads.end());
    for (size_t c = 0; c < m.cells.size(); ++c)
        for (int fc = 0; fc < 6; ++fc) {
            std::array<int64_t, 4> key;
            for (int v = 0; v < 4; ++v) key[v] = m.cells[c][kFaceVerts[fc][v]];
            std::sort(key.begin(), key.end());
            auto it = qmap.find(key);
            if (it != qmap.end()) m.face_bid[c][fc] = it->second;
        }
    return m;
}

// ===================================================================== mapping + metrics

namespace {

// the side of the nose cylinder's separating plane a cell lies on: the sign of
// axis . (vertex average - separation point) (manifolds/nose_cylinder.cc:45-77); 0 on the plane
int nose_side(const HexMesh& m, int64_t c)
{
    double ctr[3] = {0, 0, 0};
    for (int v = 0; v < 8; ++v)
        for (int d = 0; d < 3; ++d) ctr[d] += 0.125 * m.vertices[m.cells[c][v]][d];
    double dp = 0;
    for (int d = 0; d < 3; ++d) dp += m.axis_dir[d] * (ctr[d] - m.axis_point[d]);
    return (dp > 0) ? 1 : (dp < 0) ? -1 : 0;
}

// Physical point of reference coordinate xi in cell c through the mesh manifold. Straight cells:
// trilinear (MappingQGeneric(1)). Cylinder manifold: trilinear in cylindrical coordinates about
// the axis, which places every point on the cylindrical surfaces the vertices lie on; this stands
// in for deal.II's CylindricalManifold::get_new_point used when MappingQGeneric(m) places its
// support points (manifolds/cylinder.cc:15-33, dgsem/plens.cc:746-797). Nose cylinder
// (manifolds/nose_cylinder.cc:15-78): the cylinder rule about the axis through the separation
// point for cells before the separating plane; beyond it the spherical rule about the nose
// centre, standing in for SphericalManifold: the radius is the trilinear mean of the vertices'
// radii and the direction the normalised trilinear mean of their unit directions, which places
// every point on the spheres the vertices lie on.
std::array<double, 3> manifold_point(const HexMesh& m, int64_t c, const double xi[3])
{
    double w[8];
    for (int v = 0; v < 8; ++v) {
        const double a = (v & 1) ? xi[0] : 1 - xi[0];
        const double b = ((v >> 1) & 1) ? xi[1] : 1 - xi[1];
        const double g = ((v >> 2) & 1) ? xi[2] : 1 - xi[2];
        w[v] = a * b * g;
    }
    std::array<double, 3> out{{0, 0, 0}};
    if (m.manifold == 0) {
        for (int v = 0; v < 8; ++v)
            for (int d = 0; d < 3; ++d) out[d] += w[v] * m.vertices[m.cells[c][v]][d];
        return out;
    }
    if (m.manifold == 2 && nose_side(m, c) > 0) {
        double rr = 0, dir[3] = {0, 0, 0};
        for (int v = 0; v < 8; ++v) {
            const auto& p = m.vertices[m.cells[c][v]];
            const double q[3] = {p[0] - m.nose_center[0], p[1] - m.nose_center[1], p[2] - m.nose_center[2]};
            const double r = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            rr += w[v] * r;
            for (int d = 0; d < 3; ++d) dir[d] += w[v] * q[d] / r;
        }
        const double dn = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        for (int d = 0; d < 3; ++d) out[d] = m.nose_center[d] + rr * dir[d] / dn;
        return out;
    }
    // cylinder: orthonormal frame (e1, e2, axis)
    double ax[3] = {m.axis_dir[0], m.axis_dir[1], m.axis_dir[2]};
    const double an = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    for (double& a : ax) a /= an;
    double e1[3] = {1, 0, 0};
    if (std::fabs(ax[0]) > 0.9) { e1[0] = 0; e1[1] = 1; }
    const double dp = e1[0] * ax[0] + e1[1] * ax[1] + e1[2] * ax[2];
    for (int d = 0; d < 3; ++d) e1[d] -= dp * ax[d];
    const double n1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (double& e : e1) e /= n1;
    const double e2[3] = {ax[1] * e1[2] - ax[2] * e1[1], ax[2] * e1[0] - ax[0] * e1[2],
                          ax[0] * e1[1] - ax[1] * e1[0]};
    double rr = 0, th = 0, aa = 0, th0 = 0;
    for (int v = 0; v < 8; ++v) {
        const auto& p = m.vertices[m.cells[c][v]];
        const double q[3] = {p[0] - m.axis_point[0], p[1] - m.axis_point[1], p[2] - m.axis_point[2]};
        const double u = q[0] * e1[0] + q[1] * e1[1] + q[2] * e1[2];
        const double s = q[0] * e2[0] + q[1] * e2[1] + q[2] * e2[2];
        const double h = q[0] * ax[0] + q[1] * ax[1] + q[2] * ax[2];
        double t = std::atan2(s, u);
        if (v == 0) th0 = t;
        while (t - th0 > M_PI) t -= 2 * M_PI;
        while (t - th0 < -M_PI) t += 2 * M_PI;
        rr += w[v] * std::sqrt(u * u + s * s);
        th += w[v] * t;
        aa += w[v] * h;
    }
    for (int d = 0; d < 3; ++d)
        out[d] = m.axis_point[d] + rr * (std::cos(th) * e1[d] + std::sin(th) * e2[d]) + aa * ax[d];
    return out;
}

}  // namespace

// ========================================================================== parameters

void declare_parameters(ParameterHandler& prm)
{
    // mesh (dgsem/plens.cc:78-152)
    prm.declare_entry("mesh/type", "straight", "straight|curved");
    prm.declare_entry("mesh/format", "msh", "msh|builtin");
    prm.declare_entry("mesh/file name", "", "mesh file (msh 2.2 ASCII)");
    prm.declare_entry("mesh/curved subtype", "cylinder", "cylinder|nose cylinder");
    prm.declare_entry("mesh/cylinder/axis direction", "1 0 0");
    prm.declare_entry("mesh/cylinder/axis point", "0 0 0");
    prm.declare_entry("mesh/nose cylinder/axis direction", "1 0 0");
    prm.declare_entry("mesh/nose cylinder/separation point", "0 0 0");
    prm.declare_entry("mesh/nose cylinder/nose center", "0 0 0");
    prm.declare_entry("mesh/builtin/generator", "box", "box|o-mesh (replaces gmsh for generated meshes)");
    prm.declare_entry("mesh/builtin/lower corner", "0 0 0");
    prm.declare_entry("mesh/builtin/upper corner", "1 1 1");
    prm.declare_entry("mesh/builtin/subdivisions", "1 1 1");
    prm.declare_entry("mesh/builtin/boundary ids", "1 2 3 4 5 6", "ids of the -x,+x,-y,+y,-z,+z sides");
    prm.declare_entry("mesh/builtin/split -y side at x", "none", "faces of the -y side beyond this x get 'split boundary id'");
    prm.declare_entry("mesh/builtin/split boundary id", "7");
    prm.declare_entry("mesh/builtin/inner radius", "1");
    prm.declare_entry("mesh/builtin/outer radius", "10");
    prm.declare_entry("mesh/builtin/radial cells", "16");
    prm.declare_entry("mesh/builtin/azimuthal cells", "16");
    prm.declare_entry("mesh/builtin/first cell height", "1e-3");
    prm.declare_entry("mesh/builtin/z cells", "1");
    prm.declare_entry("mesh/builtin/z length", "0.1");
    prm.declare_entry("mesh/builtin/o-mesh boundary ids", "1 2 3 4 5", "inner, outer x<0, outer x>0, -z, +z");
    // Navier-Stokes (dgsem/plens.cc:154-250)
    prm.declare_entry("Navier-Stokes/gas name", "air", "air|nitrogen|custom");
    prm.declare_entry("Navier-Stokes/inviscid", "true");
    prm.declare_entry("Navier-Stokes/gamma", "1.4");
    prm.declare_entry("Navier-Stokes/molecular weight", "0.028");
    prm.declare_entry("Navier-Stokes/Prandtl number", "0.71");
    prm.declare_entry("Navier-Stokes/mu0", "1e-5");
    prm.declare_entry("Navier-Stokes/T0", "300");
    prm.declare_entry("Navier-Stokes/S", "100");
    prm.declare_entry("Navier-Stokes/auxiliary surface flux scheme", "BR1");
    prm.declare_entry("Navier-Stokes/auxiliary volume flux scheme", "BR1");
    prm.declare_entry("Navier-Stokes/inviscid surface flux scheme", "Chandrashekhar");
    prm.declare_entry("Navier-Stokes/inviscid volume flux scheme", "Chandrashekhar");
    prm.declare_entry("Navier-Stokes/diffusive surface flux scheme", "BR1");
    prm.declare_entry("Navier-Stokes/diffusive volume flux scheme", "BR1");
    // BCs (dgsem/plens.cc:252-320)
    for (int i = 1; i <= 12; ++i) {
        const std::string b = "BCs/bid" + std::to_string(i) + "/";
        prm.declare_entry(b + "type", "none");
        prm.declare_entry(b + "prescribed p", "1e5");
        prm.declare_entry(b + "prescribed T", "1");
        prm.declare_entry(b + "prescribed velocity", "0 0 0");
        prm.declare_entry(b + "periodic direction", "0");
        prm.declare_entry(b + "periodic orientation", "left");
        prm.declare_entry(b + "other surface boundary id", "1");
    }
    // IC (dgsem/plens.cc:322-380) + the seeded perturbations of this build's configs
    prm.declare_entry("IC/type", "piecewise function",
                      "piecewise function|double mach reflection|uniform|shock vortex|from archive restart");
    prm.declare_entry("IC/file name", "ic.dat");
    prm.declare_entry("IC/archive mesh file name", "mesh.msh");
    prm.declare_entry("IC/archive mesh format", "msh");
    prm.declare_entry("IC/archive fe degree", "1");
    prm.declare_entry("IC/double mach reflection/wedge leading edge location", "0.16666667 0 0");
    prm.declare_entry("IC/double mach reflection/wedge angle", "0");
    prm.declare_entry("IC/double mach reflection/shock offset", "0 0 0");
    prm.declare_entry("IC/uniform/primitive state", "1 0 0 0 1", "rho u v w p");
    prm.declare_entry("IC/uniform/wall damping radius", "0",
                      "if > 0: the velocity is scaled by 1-exp(-(r-R)/L), r = distance from the z axis");
    prm.declare_entry("IC/uniform/wall damping length", "0.5");
    prm.declare_entry("IC/shock vortex/turbulent Mach number", "0.6");
    prm.declare_entry("IC/shock vortex/shock Mach number", "3");
    prm.declare_entry("IC/shock vortex/shock x", "3.14159265358979");
    prm.declare_entry("IC/shock vortex/modes", "8", "wavenumbers per direction in the random-phase field");
    prm.declare_entry("IC/noise/variable", "none", "none|rho|pre-shock rho|velocity");
    prm.declare_entry("IC/noise/amplitude", "0");
    prm.declare_entry("IC/noise/seed", "1");
    // blender parameters (dgsem/plens.cc:400-510)
    prm.declare_entry("blender parameters/variable", "pxrho");
    prm.declare_entry("blender parameters/blender function", "Hennemann");
    prm.declare_entry("blender parameters/threshold factor", "0.5");
    prm.declare_entry("blender parameters/threshold exponent factor", "1.8");
    prm.declare_entry("blender parameters/sharpness factor", "9.21024");
    prm.declare_entry("blender parameters/blender min value", "1e-3");
    prm.declare_entry("blender parameters/blender max value", "0.5");
    prm.declare_entry("blender parameters/wall blender limit", "0.5");
    prm.declare_entry("blender parameters/viscous blending region", "1");
    prm.declare_entry("blender parameters/do filtering", "false");
    // time integration (dgsem/plens.cc:512-582)
    prm.declare_entry("time integration/RK order", "4");
    prm.declare_entry("time integration/Courant number", "0.1");
    prm.declare_entry("time integration/start time", "0");
    prm.declare_entry("time integration/starting output counter", "0");
    prm.declare_entry("time integration/end time", "1");
    prm.declare_entry("time integration/request local stepping", "false");
    prm.declare_entry("time integration/local stepping start time", "100");
    prm.declare_entry("time integration/limit local time step", "false");
    prm.declare_entry("time integration/local step neighbor factor", "1.05");
    prm.declare_entry("time integration/local step global factor", "1000");
    // data output (dgsem/plens.cc:584-644)
    prm.declare_entry("data output/directory", "result");
    prm.declare_entry("data output/base file name", "output");
    prm.declare_entry("data output/write frequency", "100");
    prm.declare_entry("data output/calculate steady state error", "true");
    prm.declare_entry("data output/convergence/calculate error", "false");
    prm.declare_entry("data output/convergence/variable", "density");
    prm.declare_entry("data output/convergence/exact solution", "1");
    // this build: the compile-time switches of the reference as run-time options, precision
    // and the learned sensor
    prm.declare_entry("GB300/precision", "fp64", "fp64|mixed|mixed_r32");
    prm.declare_entry("GB300/sensor", "modal", "modal|learned");
    prm.declare_entry("GB300/sensor weights file", "");
    prm.declare_entry("GB300/judge every", "25");
    prm.declare_entry("GB300/judge alpha tolerance", "0.05");
    prm.declare_entry("GB300/constant viscosity", "false", "CONST_VISCOSITY build switch");
    prm.declare_entry("GB300/2d", "false", "PLENS_2D build switch");
    prm.declare_entry("GB300/geometry setup", "host", "host|gpu: where the metric terms and face dofs are computed");
}

void prim_to_cons(double gamma, double rho, const double vel[3], double p, double cons[5])
{
    cons[0] = rho;
    cons[4] = p / (gamma - 1);
    for (int d = 0; d < 3; ++d) {
        cons[1 + d] = rho * vel[d];
        cons[4] += 0.5 * rho * vel[d] * vel[d];
    }
}

void Case::finalize_pointers()
{
    mesh.degree = degree;
    mesh.n_cells = n_cells;
    mesh.detJ = detJ.data();
    mesh.Ja = Ja.data();
    mesh.Jinv = Jinv.data();
    mesh.h_min = h_min.data();
    mesh.cell_center = cell_center.data();
    mesh.cell_nbr = cell_nbr.data();
    mesh.cell_face_bc = cell_face_bc.data();
    mesh.n_face_tasks = static_cast<int64_t>(ft_cell.size());
    mesh.ft_cell = ft_cell.data();
    mesh.ft_face = ft_face.data();
    mesh.ft_nbr_cell = ft_nbr_cell.data();
    mesh.ft_nbr_face = ft_nbr_face.data();
    mesh.ft_bc = ft_bc.data();
    mesh.ft_nbr_fdof = ft_nbr_fdof.data();
    mesh.ft_normal = ft_normal.data();
    mesh.ft_xyz = ft_xyz.data();
    mesh.gauss_interp = gauss_interp.empty() ? nullptr : gauss_interp.data();
    mesh.q_wJ = q_wJ.empty() ? nullptr : q_wJ.data();
    mesh.q_xyz = q_xyz.empty() ? nullptr : q_xyz.data();
    params.n_bc = static_cast<int32_t>(bcs.size());
    params.bcs = bcs.data();
    params.n_expr = exprs.size();
    params.expr_offset = exprs.offset.data();
    params.expr_length = exprs.length.data();
    params.n_expr_insn = static_cast<int32_t>(exprs.code.size());
    params.expr_code = exprs.code.data();
}

namespace {

std::array<double, 3> parse3(const std::string& s, const std::string& what)
{
    auto v = split_string(s, " ");
    if (v.size() != 3) throw std::runtime_error(what + " needs 3 numbers: '" + s + "'");
    return {std::stod(v[0]), std::stod(v[1]), std::stod(v[2])};
}

// face-local dof -> cell-local dof (dgsem/face_dof_info.h:92-150)
int face_to_cell_dof(int P, int face, int q)
{
    const int a = q % P, b = q / P;
    switch (face) {
    case 0: return P * q;                      // (0, a, b)
    case 1: return (P - 1) + P * q;            // (N, a, b)
    case 2: return a + P * P * b;              // (a, 0, b): x fastest then z
    case 3: return a + P * (P - 1) + P * P * b;
    case 4: return q;                          // (a, b, 0)
    default: return q + P * P * (P - 1);       // (a, b, N)
    }
}

// The cell-local node at which FEFaceValues::normal_vector(q) is evaluated for face `face`.
// FEFaceValues numbers face quadrature points through QProjector, whose face coordinate systems
// are (y,z) on faces 0/1, (z,x) on faces 2/3 and (x,y) on faces 4/5; the face dofs of
// face_dof_info.h run x fastest on faces 2/3. dgsem/plens.cc:1790-1797 indexes both with the same
// q, so on faces 2/3 the normal of the transposed node is used. This is reproduced; it has no
// effect where those faces are planar (every mesh this build generates).
int normal_node_of_face_dof(int P, int face, int q)
{
    if (face == 2 || face == 3) {
        const int qt = (q % P) * P + (q / P);
        return face_to_cell_dof(P, face, qt);
    }
    return face_to_cell_dof(P, face, q);
}

// Support points of MappingQGeneric(m) for every cell: the manifold point at each tensor point of
// the 1D support nodes xi_s, [n_cells][M1^3][3] with point i + M1 (j + M1 k).
std::vector<double> support_points(const HexMesh& mesh, const std::vector<double>& xi_s)
{
    const int M1 = static_cast<int>(xi_s.size()), M3 = M1 * M1 * M1;
    const int64_t nc = static_cast<int64_t>(mesh.cells.size());
    std::vector<double> sup(static_cast<size_t>(nc) * M3 * 3);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nc; ++c)
        for (int k = 0; k < M1; ++k)
            for (int j = 0; j < M1; ++j)
                for (int i = 0; i < M1; ++i) {
                    const double xi[3] = {xi_s[i], xi_s[j], xi_s[k]};
                    const auto p = manifold_point(mesh, c, xi);
                    for (int d = 0; d < 3; ++d) sup[(static_cast<size_t>(c) * M3 + i + M1 * (j + M1 * k)) * 3 + d] = p[d];
                }
    return sup;
}

// Host form of plens_gpu_setup_geometry (include/plens_gpu.h), the same job in the same
// arithmetic: MetricTerms<3>::reinit at the nodes of a tensor rule (dgsem/metric_terms.cc:67-142:
// J from the mapping, det J, J^-1 by cofactors, Ja^d = a_{d+1} x a_{d+2}) and the face-dof
// matching of form_neighbor_face_matchings (dgsem/plens.cc:1574-1627) with the unit normals of
// FEFaceValues (dgsem/plens.cc:1751-1756, 1797).
int host_setup_geometry(plens_geometry_job* jb)
{
    const int np = jb->n_points, ns = jb->n_support, np2 = np * np, np3 = np2 * np, ns3 = ns * ns * ns;
    const int64_t nc = jb->n_cells, nn = nc * np3;
    const double* Ls = jb->basis;
    const double* dLs = jb->dbasis;
    std::vector<double> xyz_tmp, ja_tmp;
    double* xyz = jb->xyz;
    double* Ja = jb->Ja;
    if (jb->n_face_tasks > 0 && (!xyz || !Ja)) return PLENS_GPU_E_INVALID;
    int64_t bad = INT64_MAX;
#pragma omp parallel for schedule(static) reduction(min : bad)
    for (int64_t c = 0; c < nc; ++c) {
        const double* sup = jb->support + static_cast<size_t>(c) * ns3 * 3;
        for (int l = 0; l < np3; ++l) {
            const int ti[3] = {l % np, (l / np) % np, l / np2};
            double x[3] = {0, 0, 0}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int k = 0; k < ns; ++k)
                for (int j = 0; j < ns; ++j)
                    for (int i = 0; i < ns; ++i) {
                        const double* X = sup + (i + ns * (j + ns * k)) * 3;
                        const double li = Ls[ti[0] * ns + i], lj = Ls[ti[1] * ns + j], lk = Ls[ti[2] * ns + k];
                        const double g[3] = {dLs[ti[0] * ns + i] * lj * lk, li * dLs[ti[1] * ns + j] * lk,
                                             li * lj * dLs[ti[2] * ns + k]};
                        for (int d = 0; d < 3; ++d) {
                            x[d] += X[d] * li * lj * lk;
                            for (int e = 0; e < 3; ++e) J[d][e] += X[d] * g[e];
                        }
                    }
            const int64_t node = c * np3 + l;
            if (xyz)
                for (int d = 0; d < 3; ++d) xyz[d * nn + node] = x[d];
            const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
            if (!(det > 0)) bad = std::min(bad, c);
            if (jb->detJ) jb->detJ[node] = det;
            if (jb->Jinv) {
                double inv[3][3];
                inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
                inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
                inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
                inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
                inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
                inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
                inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
                inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
                inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
                for (int r = 0; r < 3; ++r)
                    for (int cc = 0; cc < 3; ++cc) jb->Jinv[(r * 3 + cc) * nn + node] = inv[r][cc];
            }
            // covariant vectors a_d = column d of J; Ja^d = a_{d+1} x a_{d+2}
            if (Ja)
                for (int d = 0; d < 3; ++d) {
                    const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
                    const double a1[3] = {J[0][d1], J[1][d1], J[2][d1]};
                    const double a2[3] = {J[0][d2], J[1][d2], J[2][d2]};
                    const double cr[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2],
                                          a1[0] * a2[1] - a1[1] * a2[0]};
                    for (int e = 0; e < 3; ++e) Ja[(d * 3 + e) * nn + node] = cr[e];
                }
        }
    }
    jb->first_bad_cell = (bad == INT64_MAX) ? -1 : bad;

    // face dofs: the first face dof of the other side within the tolerance (periodic direction
    // left out of the distance), the unit outward normal at the node FEFaceValues uses, the location
    const int64_t nt = jb->n_face_tasks;
    int64_t unmatched = INT64_MAX, misoriented = INT64_MAX;
#pragma omp parallel for schedule(static) reduction(min : unmatched, misoriented)
    for (int64_t t = 0; t < nt; ++t) {
        const int64_t c = jb->ft_cell[t], oc = jb->ft_nbr_cell[t];
        const int f = jb->ft_face[t], of = jb->ft_nbr_face[t], pdir = jb->ft_skip_dir[t];
        const double tol = jb->ft_tol[t];
        for (int q = 0; q < np2; ++q) {
            const int64_t idx = t * np2 + q;
            const int64_t own = c * np3 + face_to_cell_dof(np, f, q);
            int match = (oc < 0) ? q : -1;
            if (oc >= 0) {
                for (int q2 = 0; q2 < np2 && match < 0; ++q2) {
                    const int64_t other = oc * np3 + face_to_cell_dof(np, of, q2);
                    double s2 = 0;
                    for (int d = 0; d < 3; ++d) {
                        if (d == pdir) continue;
                        const double df = xyz[d * nn + own] - xyz[d * nn + other];
                        s2 += df * df;
                    }
                    if (std::sqrt(s2) < tol) match = q2;
                }
                if (match < 0) unmatched = std::min(unmatched, idx);
                else if (pdir >= 0 && match != q) misoriented = std::min(misoriented, idx);
            }
            jb->ft_nbr_fdof[idx] = match;
            const int64_t ln = c * np3 + normal_node_of_face_dof(np, f, q);
            const int dir = f / 2;
            const double sgn = (f % 2 == 0) ? -1.0 : 1.0;
            double n[3], nrm = 0;
            for (int e = 0; e < 3; ++e) {
                n[e] = Ja[(dir * 3 + e) * nn + ln];
                nrm += n[e] * n[e];
            }
            nrm = std::sqrt(nrm);
            for (int e = 0; e < 3; ++e) jb->ft_normal[idx * 3 + e] = sgn * n[e] / nrm;
            for (int e = 0; e < 3; ++e) jb->ft_xyz[idx * 3 + e] = xyz[e * nn + own];
        }
    }
    jb->first_unmatched = (unmatched == INT64_MAX) ? -1 : unmatched;
    jb->first_misoriented = (misoriented == INT64_MAX) ? -1 : misoriented;
    return PLENS_GPU_OK;
}

}  // namespace

std::unique_ptr<Case> build_case(const ParameterHandler& prm, int mapping_degree, int fe_degree,
                                 const std::string& base_dir, plens_geometry_fn geometry)
{
    auto cs = std::make_unique<Case>();
    Case& C = *cs;
    auto clock_now = [] { return std::chrono::steady_clock::now(); };
    auto lap = clock_now();
    auto charge = [&](int phase) {
        const auto t = clock_now();
        C.setup_seconds[phase] += std::chrono::duration<double>(t - lap).count();
        lap = t;
    };
    if (fe_degree < 1 || fe_degree > 5) throw std::runtime_error("fe degree must lie in [1,5]");
    if (mapping_degree < 1) throw std::runtime_error("High order mapping degree must be >= 1.");
    C.degree = fe_degree;
    const int P = fe_degree + 1, P2 = P * P, P3 = P2 * P;
    auto path = [&](const std::string& f) {
        if (f.empty() || f[0] == '/' || base_dir.empty()) return f;
        return base_dir + "/" + f;
    };

    // ------------------------------------------------------------ read_mesh (plens.cc:699-803)
    HexMesh mesh;
    const std::string mtype = prm.get("mesh/type"), mformat = prm.get("mesh/format");
    if (mformat == "builtin") {
        const std::string gen = prm.get("mesh/builtin/generator");
        if (gen == "box") {
            BoxSpec b;
            b.lo = parse3(prm.get("mesh/builtin/lower corner"), "lower corner");
            b.hi = parse3(prm.get("mesh/builtin/upper corner"), "upper corner");
            auto n = parse3(prm.get("mesh/builtin/subdivisions"), "subdivisions");
            for (int d = 0; d < 3; ++d) b.n[d] = static_cast<int>(n[d]);
            auto ids = split_string(prm.get("mesh/builtin/boundary ids"), " ");
            if (ids.size() != 6) throw std::runtime_error("box needs 6 boundary ids");
            for (int f = 0; f < 6; ++f) b.bid[f] = std::stoi(ids[f]);
            const std::string sp = prm.get("mesh/builtin/split -y side at x");
            if (sp != "none") {
                b.split = true;
                b.split_x = std::stod(sp);
                b.split_bid = static_cast<int32_t>(prm.get_integer("mesh/builtin/split boundary id"));
            }
            mesh = make_box(b);
        } else if (gen == "o-mesh") {
            OMeshSpec o;
            o.r_inner = prm.get_double("mesh/builtin/inner radius");
            o.r_outer = prm.get_double("mesh/builtin/outer radius");
            o.n_radial = static_cast<int>(prm.get_integer("mesh/builtin/radial cells"));
            o.n_azimuthal = static_cast<int>(prm.get_integer("mesh/builtin/azimuthal cells"));
            o.first_cell = prm.get_double("mesh/builtin/first cell height");
            o.n_z = static_cast<int>(prm.get_integer("mesh/builtin/z cells"));
            o.z_length = prm.get_double("mesh/builtin/z length");
            auto ids = split_string(prm.get("mesh/builtin/o-mesh boundary ids"), " ");
            if (ids.size() != 5) throw std::runtime_error("o-mesh needs 5 boundary ids");
            o.bid_inner = std::stoi(ids[0]);
            o.bid_outer_front = std::stoi(ids[1]);
            o.bid_outer_back = std::stoi(ids[2]);
            o.bid_zlo = std::stoi(ids[3]);
            o.bid_zhi = std::stoi(ids[4]);
            mesh = make_o_mesh(o);
        } else {
            throw std::runtime_error("unknown builtin mesh generator " + gen);
        }
    } else if (mformat == "msh") {
        mesh = read_msh(path(prm.get("mesh/file name")));
    } else {
        throw std::runtime_error("mesh format '" + mformat + "' is not supported (msh|builtin)");
    }
    if (mtype == "straight") {
        mesh.manifold = 0;
        C.mapping_degree = 1;
    } else if (mtype == "curved") {
        const std::string sub = prm.get("mesh/curved subtype");
        if (sub == "cylinder") {
            mesh.manifold = 1;
            mesh.axis_dir = parse3(prm.get("mesh/cylinder/axis direction"), "axis direction");
            mesh.axis_point = parse3(prm.get("mesh/cylinder/axis point"), "axis point");
        } else if (sub == "nose cylinder") {
            // manifolds/nose_cylinder.cc:15-78 and the reading of its parameters (plens.cc:746-797)
            mesh.manifold = 2;
            mesh.axis_dir = parse3(prm.get("mesh/nose cylinder/axis direction"), "axis direction");
            mesh.axis_point = parse3(prm.get("mesh/nose cylinder/separation point"), "separation point");
            mesh.nose_center = parse3(prm.get("mesh/nose cylinder/nose center"), "nose center");
            double dp = 0;
            for (int d = 0; d < 3; ++d) dp += mesh.axis_dir[d] * (mesh.nose_center[d] - mesh.axis_point[d]);
            if (!(dp < 0))
                throw std::runtime_error("The nose center lies in spherical region. This will produce a singularity in "
                                         "spherical manifold.");
            for (int64_t c = 0; c < (int64_t)mesh.cells.size(); ++c)
                if (nose_side(mesh, c) == 0)
                    throw std::runtime_error("One of the cell centers in the triangulation provided lies on the "
                                             "bifurcation plane (cell " + std::to_string(c) + ").");
        } else {
            throw std::runtime_error("curved subtype must be cylinder|nose cylinder");
        }
        C.mapping_degree = mapping_degree;
    } else {
        throw std::runtime_error("mesh type must be straight|curved");
    }
    const int64_t nc = static_cast<int64_t>(mesh.cells.size());
    if (nc == 0) throw std::runtime_error("mesh has no cells");
    C.n_cells = nc;
    C.n_dofs = nc * P3;
    const int64_t nd = C.n_dofs;

    // ---------------------------------------------------- set_NS (plens.cc:811-885)
    plens_params& pr = C.params;
    pr.degree = fe_degree;
    {
        const std::string gas = prm.get("Navier-Stokes/gas name");
        const double R0 = 8.314462618;
        double M;
        if (gas == "custom") {
            pr.gamma = prm.get_double("Navier-Stokes/gamma");
            M = prm.get_double("Navier-Stokes/molecular weight");
            pr.Pr = prm.get_double("Navier-Stokes/Prandtl number");
            pr.mu0 = prm.get_double("Navier-Stokes/mu0");
            pr.T0 = prm.get_double("Navier-Stokes/T0");
            pr.S = prm.get_double("Navier-Stokes/S");
        } else if (gas == "air" || gas == "nitrogen" || gas == "N2") {
            // NavierStokes(gas_name, inviscid) (navier_stokes.cc:48-82)
            const bool inv = prm.get_bool("Navier-Stokes/inviscid");
            pr.gamma = 1.4;
            pr.Pr = 0.69;
            pr.T0 = 273;
            if (gas == "air") { M = 0.029; pr.mu0 = inv ? 0 : 1.716e-5; pr.S = 111; }
            else { M = 0.028; pr.mu0 = inv ? 0 : 1.663e-5; pr.S = 107; }
        } else {
            throw std::runtime_error("Unsupported gas name " + gas);
        }
        pr.R = R0 / M;
        const std::string isfs = prm.get("Navier-Stokes/inviscid surface flux scheme");
        static const std::map<std::string, int> isf = {
            {"HLLC", PLENS_ISF_HLLC}, {"Rusanov", PLENS_ISF_RUSANOV},
            {"AUSM+-up", PLENS_ISF_AUSM_PLUS_UP}, {"Rusanov-HLLC", PLENS_ISF_RUSANOV_HLLC},
            {"Rusanov-AUSM+-up", PLENS_ISF_RUSANOV_AUSM_PLUS_UP}, {"Modified SW", PLENS_ISF_MODIFIED_SW},
            {"Chandrashekhar", PLENS_ISF_CHANDRASHEKHAR}, {"KG", PLENS_ISF_KENNEDY_GRUBER},
            {"Rusanov-KG", PLENS_ISF_RUSANOV_KENNEDY_GRUBER}, {"IR", PLENS_ISF_ISMAIL_ROE}};
        auto it = isf.find(isfs);
        // "SLAU2" is not accepted: the reference's set_NS leaves the scheme unset for it (the
        // assignment is written as a comparison, dgsem/plens.cc:845)
        if (it == isf.end()) throw std::runtime_error("unsupported inviscid surface flux scheme " + isfs);
        pr.inv_surf_flux = it->second;
        const std::string ivfs = prm.get("Navier-Stokes/inviscid volume flux scheme");
        if (ivfs == "Chandrashekhar") pr.inv_vol_flux = PLENS_IVF_CHANDRASHEKHAR;
        else if (ivfs == "KG") pr.inv_vol_flux = PLENS_IVF_KENNEDY_GRUBER;
        else if (ivfs == "IR") pr.inv_vol_flux = PLENS_IVF_ISMAIL_ROE;
        else throw std::runtime_error("unsupported inviscid volume flux scheme " + ivfs);
        pr.const_viscosity = prm.get_bool("GB300/constant viscosity") ? 1 : 0;
        pr.plens_2d = prm.get_bool("GB300/2d") ? 1 : 0;
    }

    // ------------------------------------------- blender + time settings (plens.cc:1447-1499)
    {
        const std::string var = prm.get("blender parameters/variable");
        pr.blender_variable = (var == "pxrho") ? 0 : (var == "p") ? 1 : (var == "rho") ? 2 : -1;
        if (pr.blender_variable < 0) throw std::runtime_error("blender variable must be pxrho|p|rho");
        const std::string fn = prm.get("blender parameters/blender function");
        if (fn == "Hennemann") pr.blender_function = 0;
        else if (fn == "linear") pr.blender_function = 1;
        else throw std::runtime_error("custom blender functions are not supported: " + fn);
        pr.threshold_factor = prm.get_double("blender parameters/threshold factor");
        pr.threshold_exp_factor = prm.get_double("blender parameters/threshold exponent factor");
        pr.sharpness_factor = prm.get_double("blender parameters/sharpness factor");
        pr.alpha_min = prm.get_double("blender parameters/blender min value");
        pr.alpha_max = prm.get_double("blender parameters/blender max value");
        pr.expr_wall_blender_limit = C.exprs.add(prm.get("blender parameters/wall blender limit"));
        pr.expr_vis_blending_region = C.exprs.add(prm.get("blender parameters/viscous blending region"));
        pr.do_filtering = prm.get_bool("blender parameters/do filtering") ? 1 : 0;
        pr.rk_order = static_cast<int32_t>(prm.get_integer("time integration/RK order"));
        if (pr.rk_order != 3 && pr.rk_order != 4) throw std::runtime_error("RK order must be 3 or 4");
        pr.expr_courant = C.exprs.add(prm.get("time integration/Courant number"));
        C.start_time = prm.get_double("time integration/start time");
        C.end_time = prm.get_double("time integration/end time");
        C.starting_output_counter = prm.get_integer("time integration/starting output counter");
        pr.local_stepping = prm.get_bool("time integration/request local stepping") ? 1 : 0;
        pr.local_start_time = prm.get_double("time integration/local stepping start time");
        pr.limit_local_step = prm.get_bool("time integration/limit local time step") ? 1 : 0;
        pr.local_nbr_factor = prm.get_double("time integration/local step neighbor factor");
        pr.local_global_factor = prm.get_double("time integration/local step global factor");
        pr.calc_ss_error = prm.get_bool("data output/calculate steady state error") ? 1 : 0;
        pr.calc_conv_error = prm.get_bool("data output/convergence/calculate error") ? 1 : 0;
        pr.expr_conv_exact = -1;
        if (pr.calc_conv_error) {
            if (prm.get("data output/convergence/variable") != "density")
                throw std::runtime_error("Currently, only density variable is supported for convergence error calculation.");
            pr.expr_conv_exact = C.exprs.add(prm.get("data output/convergence/exact solution"));
        }
        C.write_freq = prm.get_integer("data output/write frequency");
        C.output_dir = prm.get("data output/directory");
        C.base_file_name = prm.get("data output/base file name");
        const std::string prec = prm.get("GB300/precision");
        pr.precision = (prec == "mixed") ? PLENS_PRECISION_MIXED : (prec == "mixed_r32") ? PLENS_PRECISION_MIXED_R32 : PLENS_PRECISION_FP64;
        if (prec != "mixed" && prec != "mixed_r32" && prec != "fp64")
            throw std::runtime_error("GB300/precision must be fp64|mixed|mixed_r32");
        const std::string sens = prm.get("GB300/sensor");
        pr.sensor = (sens == "learned") ? PLENS_SENSOR_LEARNED : PLENS_SENSOR_MODAL;
        pr.judge_every = static_cast<int32_t>(prm.get_integer("GB300/judge every"));
        pr.judge_alpha_tol = prm.get_double("GB300/judge alpha tolerance");
        C.sensor_weights_file = prm.get("GB300/sensor weights file");
        if (!C.sensor_weights_file.empty()) C.sensor_weights_file = path(C.sensor_weights_file);
    }

    // ------------------------------------------------------- 1D rules, cell sizes, geometry
    std::vector<double> xi_n, w_n;
    gll_1d(P, xi_n, w_n);
    const int m_deg = C.mapping_degree, M1 = m_deg + 1;
    std::vector<double> xi_s, w_s;
    gll_1d(M1, xi_s, w_s);
    charge(0);
    C.h_min.assign(nc, 0);
    C.cell_center.assign(3 * nc, 0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nc; ++c) {
        // minimum_vertex_distance (all vertex pairs) and centre (vertex average)
        double hmin2 = 1e300;
        for (int a = 0; a < 8; ++a)
            for (int b = a + 1; b < 8; ++b) {
                double s2 = 0;
                for (int d = 0; d < 3; ++d) {
                    const double df = mesh.vertices[mesh.cells[c][a]][d] - mesh.vertices[mesh.cells[c][b]][d];
                    s2 += df * df;
                }
                hmin2 = std::min(hmin2, s2);
            }
        C.h_min[c] = std::sqrt(hmin2);
        for (int v = 0; v < 8; ++v)
            for (int d = 0; d < 3; ++d) C.cell_center[3 * c + d] += 0.125 * mesh.vertices[mesh.cells[c][v]][d];
    }
    // The geometry jobs (metric terms, face dofs) run on the host, or with "GB300/geometry setup =
    // gpu" through `geometry` (plens_gpu_setup_geometry); both give the same bits.
    const std::string geo_mode = prm.get("GB300/geometry setup");
    if (geo_mode != "host" && geo_mode != "gpu") throw std::runtime_error("GB300/geometry setup must be host|gpu");
    const bool geo_gpu = geo_mode == "gpu";
    if (geo_gpu && !geometry)
        throw std::runtime_error("GB300/geometry setup = gpu needs the GPU library's geometry function");
    auto run_job = [&](plens_geometry_job& jb) {
        const int rc = geo_gpu ? geometry(&jb) : host_setup_geometry(&jb);
        if (rc != PLENS_GPU_OK)
            throw std::runtime_error(std::string("geometry setup failed on the ") + (geo_gpu ? "GPU" : "host") +
                                     " with status " + std::to_string(rc));
    };
    const std::vector<double> sup = support_points(mesh, xi_s);
    charge(1);

    // ------------------------------------------------------------------- topology
    C.cell_nbr.assign(6 * nc, -1);
    C.cell_face_bc.assign(6 * nc, -1);
    std::vector<int32_t> nbr_face(6 * nc, -1);
    {
        std::map<std::array<int64_t, 4>, std::pair<int64_t, int>> open;
        for (int64_t c = 0; c < nc; ++c)
            for (int f = 0; f < 6; ++f) {
                std::array<int64_t, 4> key;
                for (int v = 0; v < 4; ++v) key[v] = mesh.cells[c][kFaceVerts[f][v]];
                std::sort(key.begin(), key.end());
                auto it = open.find(key);
                if (it == open.end()) {
                    open.emplace(key, std::make_pair(c, f));
                } else {
                    const int64_t c2 = it->second.first;
                    const int f2 = it->second.second;
                    C.cell_nbr[6 * c + f] = static_cast<int32_t>(c2);
                    C.cell_nbr[6 * c2 + f2] = static_cast<int32_t>(c);
                    nbr_face[6 * c + f] = f2;
                    nbr_face[6 * c2 + f2] = f;
                    open.erase(it);
                }
            }
        for (const auto& [key, cf] : open) {
            const int32_t bid = mesh.face_bid[cf.first][cf.second];
            if (bid < 0) throw std::runtime_error("boundary face without boundary id at cell " + std::to_string(cf.first));
            C.cell_face_bc[6 * cf.first + cf.second] = bid;
        }
    }

    // ------------------------------------------------------------------- set_BC
    // (plens.cc:1219-1440). Descriptors indexed by boundary id 0..12.
    C.bcs.assign(13, plens_bc_desc{});
    for (auto& b : C.bcs) {
        b.type = PLENS_BC_NONE;
        b.expr_p = b.expr_T = -1;
        b.expr_vel[0] = b.expr_vel[1] = b.expr_vel[2] = -1;
    }
    std::vector<int> used(13, 0);
    for (int64_t c = 0; c < nc; ++c)
        for (int f = 0; f < 6; ++f) {
            const int32_t b = C.cell_face_bc[6 * c + f];
            if (b >= 0) {
                if (b < 1 || b > 12) throw std::runtime_error("boundary ids must lie in 1..12");
                used[b] = 1;
            }
        }
    struct PeriodicSpec { int dir; int other; bool left; };
    std::map<int, PeriodicSpec> periodic;
    for (int b = 1; b <= 12; ++b) {
        if (!used[b]) continue;
        const std::string s = "BCs/bid" + std::to_string(b) + "/";
        const std::string type = prm.get(s + "type");
        plens_bc_desc& d = C.bcs[b];
        auto vel3 = [&]() { return parse3(prm.get(s + "prescribed velocity"), "prescribed velocity"); };
        if (type == "none") {
            throw std::runtime_error("'none' type BC is not for ids specified in the mesh (bid" + std::to_string(b) + ")");
        } else if (type == "free") {
            d.type = PLENS_BC_FREE;
        } else if (type == "outflow") {
            d.type = PLENS_BC_OUTFLOW;
            d.p = prm.get_double(s + "prescribed p");
        } else if (type == "uniform inflow") {
            d.type = PLENS_BC_UNIFORM_INFLOW;
            d.p = prm.get_double(s + "prescribed p");
            d.T = prm.get_double(s + "prescribed T");
            auto v = vel3();
            for (int k = 0; k < 3; ++k) d.vel[k] = v[k];
            prim_to_cons(pr.gamma, d.p / (pr.R * d.T), d.vel, d.p, d.cons);
        } else if (type == "symmetry") {
            d.type = PLENS_BC_SYMMETRY;
        } else if (type == "empty") {
            d.type = PLENS_BC_EMPTY;
        } else if (type == "uniform temp wall") {
            d.type = PLENS_BC_UNIFORM_TEMP_WALL;
            d.T = prm.get_double(s + "prescribed T");
            auto v = vel3();
            for (int k = 0; k < 3; ++k) d.vel[k] = v[k];
        } else if (type == "insulated wall") {
            d.type = PLENS_BC_INSULATED_WALL;
            auto v = vel3();
            for (int k = 0; k < 3; ++k) d.vel[k] = v[k];
        } else if (type == "ZPG inflow") {
            d.type = PLENS_BC_ZPG_INFLOW;
            auto v = vel3();
            for (int k = 0; k < 3; ++k) d.vel[k] = v[k];
        } else if (type == "varying inflow") {
            d.type = PLENS_BC_VARYING_INFLOW;
            d.expr_p = C.exprs.add(prm.get(s + "prescribed p"));
            d.expr_T = C.exprs.add(prm.get(s + "prescribed T"));
            auto comps = split_string(prm.get(s + "prescribed velocity"), ";");
            if (comps.size() != 3) throw std::runtime_error("varying inflow velocity needs 3 ';'-separated components");
            for (int k = 0; k < 3; ++k) d.expr_vel[k] = C.exprs.add(comps[k]);
        } else if (type == "periodic") {
            d.type = PLENS_BC_PERIODIC;
            PeriodicSpec ps;
            ps.dir = static_cast<int>(prm.get_integer(s + "periodic direction"));
            ps.other = static_cast<int>(prm.get_integer(s + "other surface boundary id"));
            ps.left = prm.get(s + "periodic orientation") == "left";
            if (ps.other == b)
                throw std::runtime_error("Two surfaces of a periodic pair of boundaries must have two different boundary ids");
            periodic[b] = ps;
        } else {
            throw std::runtime_error("Invalid boundary type '" + type + "'");
        }
    }

    // periodic partners (GridTools::collect_periodic_faces + BCs::Periodic): faces whose centres
    // coincide after removing the periodic coordinate
    std::vector<int32_t> per_cell(6 * nc, -1), per_face(6 * nc, -1);
    for (const auto& [b, ps] : periodic) {
        auto it = periodic.find(ps.other);
        if (it == periodic.end() || it->second.other != b || it->second.dir != ps.dir || it->second.left == ps.left)
            throw std::runtime_error("inconsistent periodic BC entries for bid" + std::to_string(b));
        std::vector<std::pair<int64_t, int>> mine, theirs;
        for (int64_t c = 0; c < nc; ++c)
            for (int f = 0; f < 6; ++f) {
                if (C.cell_face_bc[6 * c + f] == b) mine.emplace_back(c, f);
                if (C.cell_face_bc[6 * c + f] == ps.other) theirs.emplace_back(c, f);
            }
        std::map<std::pair<long long, long long>, std::pair<int64_t, int>> idx;
        const double hscale = *std::min_element(C.h_min.begin(), C.h_min.end());
        auto key = [&](const std::array<double, 3>& x) {
            int a = (ps.dir + 1) % 3, bb = (ps.dir + 2) % 3;
            if (a > bb) std::swap(a, bb);
            return std::make_pair(std::llround(x[a] / (1e-6 * hscale)), std::llround(x[bb] / (1e-6 * hscale)));
        };
        for (const auto& cf : theirs) idx[key(face_center(mesh, cf.first, cf.second))] = cf;
        for (const auto& cf : mine) {
            auto jt = idx.find(key(face_center(mesh, cf.first, cf.second)));
            if (jt == idx.end()) throw std::runtime_error("periodic face without partner on bid" + std::to_string(b));
            per_cell[6 * cf.first + cf.second] = static_cast<int32_t>(jt->second.first);
            per_face[6 * cf.first + cf.second] = jt->second.second;
        }
    }

    // ------------------------------------------------------------------- face tasks
    // interior faces once from the owner (lower cell index, plens.cc:1857), boundary faces once
    // per side. The neighbour face-dof matching by node location within 1e-8 h_min (1e-6 h_min
    // across a periodic pair, the periodic direction left out) runs in the geometry job below
    // (form_neighbor_face_matchings, plens.cc:1574-1627).
    std::vector<int32_t> ft_skip_dir;
    std::vector<double> ft_tol;
    for (int64_t c = 0; c < nc; ++c)
        for (int f = 0; f < 6; ++f) {
            const int32_t nbr = C.cell_nbr[6 * c + f];
            const int32_t bc = C.cell_face_bc[6 * c + f];
            if (bc < 0 && nbr < c) continue;  // interior face owned by the other cell
            int64_t oc = -1;
            int of = -1;
            if (bc < 0) { oc = nbr; of = nbr_face[6 * c + f]; }
            else if (C.bcs[bc].type == PLENS_BC_PERIODIC) { oc = per_cell[6 * c + f]; of = per_face[6 * c + f]; }
            C.ft_cell.push_back(static_cast<int32_t>(c));
            C.ft_face.push_back(f);
            C.ft_nbr_cell.push_back(static_cast<int32_t>(oc));
            C.ft_nbr_face.push_back(of);
            C.ft_bc.push_back(bc);
            ft_tol.push_back((bc < 0 ? 1e-8 : 1e-6) * C.h_min[c]);
            ft_skip_dir.push_back((bc >= 0 && C.bcs[bc].type == PLENS_BC_PERIODIC) ? periodic.at(bc).dir : -1);
        }

    charge(2);
    // ------------------------------------------------------ metric terms and face dofs
    // calc_metric_terms (plens.cc:1646-1682) with MetricTerms<3>::reinit (metric_terms.cc:67-142):
    // J at the GLL nodes from the mapping, detJ, Jinv, Ja^i = a_j x a_k (cyclic); then the face
    // dofs of every face task with the unit outward normal at the node FEFaceValues uses.
    {
        std::vector<double> Ls(static_cast<size_t>(P) * M1), dLs(static_cast<size_t>(P) * M1);
        for (int i = 0; i < P; ++i)
            for (int s = 0; s < M1; ++s) {
                Ls[i * M1 + s] = lagrange(xi_s, s, xi_n[i]);
                dLs[i * M1 + s] = lagrange_deriv(xi_s, s, xi_n[i]);
            }
        C.detJ.assign(nd, 0);
        C.Ja.assign(9 * nd, 0);
        C.Jinv.assign(9 * nd, 0);
        C.dof_xyz.assign(3 * nd, 0);
        const int64_t nt = static_cast<int64_t>(C.ft_cell.size());
        C.ft_nbr_fdof.assign(static_cast<size_t>(nt) * P2, -1);
        C.ft_normal.assign(static_cast<size_t>(nt) * P2 * 3, 0);
        C.ft_xyz.assign(static_cast<size_t>(nt) * P2 * 3, 0);
        plens_geometry_job jb{};
        jb.n_points = P;
        jb.n_support = M1;
        jb.n_cells = nc;
        jb.support = sup.data();
        jb.basis = Ls.data();
        jb.dbasis = dLs.data();
        jb.xyz = C.dof_xyz.data();
        jb.detJ = C.detJ.data();
        jb.Ja = C.Ja.data();
        jb.Jinv = C.Jinv.data();
        jb.n_face_tasks = nt;
        jb.ft_cell = C.ft_cell.data();
        jb.ft_face = C.ft_face.data();
        jb.ft_nbr_cell = C.ft_nbr_cell.data();
        jb.ft_nbr_face = C.ft_nbr_face.data();
        jb.ft_skip_dir = ft_skip_dir.data();
        jb.ft_tol = ft_tol.data();
        jb.ft_nbr_fdof = C.ft_nbr_fdof.data();
        jb.ft_normal = C.ft_normal.data();
        jb.ft_xyz = C.ft_xyz.data();
        run_job(jb);
        if (jb.first_bad_cell >= 0)
            throw std::runtime_error("cell " + std::to_string(jb.first_bad_cell) + " has a non-positive Jacobian");
        const int64_t um = jb.first_unmatched, mo = jb.first_misoriented;
        if (um >= 0 && (mo < 0 || um < mo)) {
            const int64_t t = um / P2;
            throw std::runtime_error("no matching face dof across face " + std::to_string(C.ft_face[t]) + " of cell " +
                                     std::to_string(C.ft_cell[t]));
        }
        if (mo >= 0) throw std::runtime_error("At least one periodic face pair doesn't have expected orientation");
    }

    // ------------------------------------------------- quadrature of the error norms
    // integrate_difference with QGauss(N+1) (dgsem/plens.cc:3985-4035, 4044-4098): per Gauss
    // point the weight times det J of the same mapping, and its location for the exact solution.
    if (C.params.calc_ss_error || C.params.calc_conv_error) {
        std::vector<double> xg, wg;
        gauss_1d(P, xg, wg);
        C.gauss_interp.assign(static_cast<size_t>(P) * P, 0);
        for (int q = 0; q < P; ++q)
            for (int i = 0; i < P; ++i) C.gauss_interp[q * P + i] = lagrange(xi_n, i, xg[q]);
        std::vector<double> Lg(static_cast<size_t>(P) * M1), dLg(static_cast<size_t>(P) * M1);
        for (int q = 0; q < P; ++q)
            for (int s = 0; s < M1; ++s) {
                Lg[q * M1 + s] = lagrange(xi_s, s, xg[q]);
                dLg[q * M1 + s] = lagrange_deriv(xi_s, s, xg[q]);
            }
        const bool want_xyz = C.params.calc_conv_error != 0;
        std::vector<double> qdet(nd);
        if (want_xyz) C.q_xyz.assign(3 * nd, 0);
        plens_geometry_job jq{};
        jq.n_points = P;
        jq.n_support = M1;
        jq.n_cells = nc;
        jq.support = sup.data();
        jq.basis = Lg.data();
        jq.dbasis = dLg.data();
        jq.xyz = want_xyz ? C.q_xyz.data() : nullptr;
        jq.detJ = qdet.data();
        run_job(jq);
        C.q_wJ.assign(nd, 0);
        for (int64_t q = 0; q < nd; ++q) {
            const int l = static_cast<int>(q % P3);
            C.q_wJ[q] = wg[l % P] * wg[(l / P) % P] * wg[l / P2] * std::fabs(qdet[q]);
        }
    }

    charge(1);
    // ------------------------------------------------------------------- set_IC
    C.U0.assign(5 * nd, 0.0);
    {
        const std::string ic = prm.get("IC/type");
        auto setU = [&](int64_t dof, const double s[5]) { for (int v = 0; v < 5; ++v) C.U0[v * nd + dof] = s[v]; };
        if (ic == "double mach reflection") {
            // ICs::DoubleMachReflection (IBCs/double_mach_reflection.cc:16-80)
            auto le = parse3(prm.get("IC/double mach reflection/wedge leading edge location"), "wedge LE");
            const double wa = prm.get_double("IC/double mach reflection/wedge angle");
            auto off = parse3(prm.get("IC/double mach reflection/shock offset"), "shock offset");
            const double sx = le[0] + off[0], sy = le[1] + off[1];
            const double cot = 1.0 / std::tan((60 + wa) * M_PI / 180);
            const double uu = 7.144709581221619, vv = 4.125;
            for (int64_t dof = 0; dof < nd; ++dof) {
                const double x = C.dof_xyz[dof], y = C.dof_xyz[nd + dof];
                if ((x - sx) - (y - sy) * cot > 0) {
                    const double s[5] = {1.4, 0, 0, 0, 1 / 0.4};
                    setU(dof, s);
                } else {
                    const double s[5] = {8, 8 * uu, -8 * vv, 0, 116.5 / 0.4 + 0.5 * 8 * (uu * uu + vv * vv)};
                    setU(dof, s);
                }
            }
        } else if (ic == "piecewise function") {
            // ICs::PiecewiseFunction (IBCs/piecewise_function.cc:31-247)
            std::ifstream f(path(prm.get("IC/file name")));
            if (!f.good()) throw std::runtime_error("Unable to open file provided for reading IC functions.");
            std::string line;
            std::getline(f, line);
            line = trim(line);
            if (line != "p" && line != "c")
                throw std::runtime_error("The first line in the file containing functions must be 'p' or 'c'");
            const bool prim = (line == "p");
            int np[3];
            for (int d = 0; d < 3; ++d) {
                std::getline(f, line);
                np[d] = static_cast<int>(std::stod(line));
                if (np[d] < 1) throw std::runtime_error("The number of pieces provided in each direction must be >= 1.");
            }
            std::vector<double> il[3];
            for (int d = 0; d < 3; ++d) {
                std::getline(f, line);
                for (const auto& sp : split_string(line, " ")) il[d].push_back(std::stod(sp));
                if (static_cast<int>(il[d].size()) != np[d] - 1)
                    throw std::runtime_error("The number of interface locations must be exactly one less than the number of pieces");
            }
            const int npieces = np[0] * np[1] * np[2];
            ExprTable fns;
            for (int pc = 0; pc < npieces * 5; ++pc) {
                if (!std::getline(f, line)) throw std::runtime_error("insufficient number of IC functions");
                fns.add(trim(line));
            }
            for (int64_t c = 0; c < nc; ++c) {
                int up[3];
                for (int d = 0; d < 3; ++d) {
                    const double xc = C.cell_center[3 * c + d];
                    up[d] = 0;
                    if (np[d] > 1) {
                        if (xc - il[d][0] < 0) up[d] = 0;
                        else if (xc - il[d][np[d] - 2] > 0) up[d] = np[d] - 1;
                        else {
                            for (int k = 0; k < np[d] - 1; ++k)
                                if (xc - il[d][k] == 0) throw std::runtime_error("The provided point lies exactly on an interface.");
                            for (int k = 1; k < np[d] - 1; ++k)
                                if (xc - il[d][k - 1] > 0 && xc - il[d][k] < 0) { up[d] = k; break; }
                        }
                    }
                }
                const int pid = up[0] + up[1] * np[0] + up[2] * np[0] * np[1];
                for (int l = 0; l < P3; ++l) {
                    const int64_t dof = c * P3 + l;
                    const double x = C.dof_xyz[dof], y = C.dof_xyz[nd + dof], z = C.dof_xyz[2 * nd + dof];
                    double v[5];
                    for (int k = 0; k < 5; ++k) v[k] = fns.eval(pid * 5 + k, x, y, z, 0);
                    if (prim) {
                        double s[5];
                        const double vel[3] = {v[1], v[2], v[3]};
                        prim_to_cons(pr.gamma, v[0], vel, v[4], s);
                        setU(dof, s);
                    } else {
                        setU(dof, v);
                    }
                }
            }
        } else if (ic == "uniform") {
            auto s = split_string(prm.get("IC/uniform/primitive state"), " ");
            if (s.size() != 5) throw std::runtime_error("uniform IC needs rho u v w p");
            const double vel[3] = {std::stod(s[1]), std::stod(s[2]), std::stod(s[3])};
            double cs5[5];
            prim_to_cons(pr.gamma, std::stod(s[0]), vel, std::stod(s[4]), cs5);
            const double Rw = prm.get_double("IC/uniform/wall damping radius");
            const double Lw = prm.get_double("IC/uniform/wall damping length");
            for (int64_t dof = 0; dof < nd; ++dof) {
                if (Rw > 0) {
                    // velocity damped to zero at the cylinder wall: an impulsive Mach 8 start
                    // empties the rear stagnation region (u > 2a/(gamma-1)), which a scheme
                    // without positivity limiting cannot represent
                    const double x = C.dof_xyz[dof], y = C.dof_xyz[nd + dof];
                    const double r = std::sqrt(x * x + y * y);
                    const double f = 1.0 - std::exp(-std::max(0.0, r - Rw) / Lw);
                    const double v2[3] = {vel[0] * f, vel[1] * f, vel[2] * f};
                    double cd[5];
                    prim_to_cons(pr.gamma, std::stod(s[0]), v2, std::stod(s[4]), cd);
                    setU(dof, cd);
                } else {
                    setU(dof, cs5);
                }
            }
        } else if (ic == "shock vortex") {
            // Random-phase solenoidal velocity field with E(k) ~ k^4 exp(-2 (k/4)^2) at turbulent
            // Mach number Mt, plus a normal shock of Mach Ms at x = xs with the Rankine-Hugoniot
            // jump behind it (post-shock state on x < xs, flow in +x). New initial condition.
            const double Mt = prm.get_double("IC/shock vortex/turbulent Mach number");
            const double Ms = prm.get_double("IC/shock vortex/shock Mach number");
            const double xs = prm.get_double("IC/shock vortex/shock x");
            const int K = static_cast<int>(prm.get_integer("IC/shock vortex/modes"));
            std::mt19937_64 rng(static_cast<uint64_t>(prm.get_integer("IC/noise/seed")));
            std::uniform_real_distribution<double> U01(0.0, 1.0);
            struct Mode { double k[3], a[3], ph; };
            std::vector<Mode> modes;
            for (int i = -K; i <= K; ++i)
                for (int j = -K; j <= K; ++j)
                    for (int l = 0; l <= K; ++l) {
                        const double kk = std::sqrt(double(i * i + j * j + l * l));
                        if (kk == 0 || kk > K) continue;
                        Mode md;
                        md.k[0] = i; md.k[1] = j; md.k[2] = l;
                        double r[3] = {U01(rng) - 0.5, U01(rng) - 0.5, U01(rng) - 0.5};
                        // project out the k component: solenoidal
                        const double dot = (r[0] * i + r[1] * j + r[2] * l) / (kk * kk);
                        double a[3] = {r[0] - dot * i, r[1] - dot * j, r[2] - dot * l};
                        const double an = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) + 1e-300;
                        const double E = std::pow(kk, 4) * std::exp(-2 * (kk / 4) * (kk / 4));
                        for (int d = 0; d < 3; ++d) md.a[d] = a[d] / an * std::sqrt(E) / kk;
                        md.ph = 2 * M_PI * U01(rng);
                        modes.push_back(md);
                    }
            std::vector<double> u(3 * nd, 0.0);
            // cos(k.x + ph) = Re(e^{i k0 x} e^{i k1 y} e^{i k2 z} e^{i ph}) with the integer
            // wavenumbers' exponentials tabulated per dof: three complex products per mode instead
            // of a cosine. The dofs are independent (threads over dofs; each dof sums its modes in
            // order), the rms is summed serially so the field does not depend on the thread count.
            std::vector<double> ph_c(modes.size()), ph_s(modes.size());
            for (size_t m = 0; m < modes.size(); ++m) {
                ph_c[m] = std::cos(modes[m].ph);
                ph_s[m] = std::sin(modes[m].ph);
            }
            // blocks of B dofs, tables [d][k][dof of block]: the innermost loop runs over the
            // block's dofs with unit stride and vectorises
            constexpr int B = 64;
            const int NK = 2 * K + 1;
            const int64_t nblk = (nd + B - 1) / B;
#pragma omp parallel
            {
                std::vector<double> ec(3 * NK * B), es(3 * NK * B), acc(3 * B);
#pragma omp for schedule(static)
                for (int64_t blk = 0; blk < nblk; ++blk) {
                    const int64_t d0 = blk * B;
                    const int nb = static_cast<int>(std::min<int64_t>(B, nd - d0));
                    for (int d = 0; d < 3; ++d)
                        for (int k = -K; k <= K; ++k)
                            for (int b = 0; b < nb; ++b) {
                                const double x = C.dof_xyz[d * nd + d0 + b];
                                ec[(d * NK + k + K) * B + b] = std::cos(k * x);
                                es[(d * NK + k + K) * B + b] = std::sin(k * x);
                            }
                    std::fill(acc.begin(), acc.end(), 0.0);
                    for (size_t m = 0; m < modes.size(); ++m) {
                        const auto& md = modes[m];
                        const double* c0 = &ec[(0 * NK + static_cast<int>(md.k[0]) + K) * B];
                        const double* s0 = &es[(0 * NK + static_cast<int>(md.k[0]) + K) * B];
                        const double* c1 = &ec[(1 * NK + static_cast<int>(md.k[1]) + K) * B];
                        const double* s1 = &es[(1 * NK + static_cast<int>(md.k[1]) + K) * B];
                        const double* c2 = &ec[(2 * NK + static_cast<int>(md.k[2]) + K) * B];
                        const double* s2 = &es[(2 * NK + static_cast<int>(md.k[2]) + K) * B];
                        const double pc = ph_c[m], ps = ph_s[m], a0 = md.a[0], a1 = md.a[1], a2 = md.a[2];
                        double* u0 = &acc[0];
                        double* u1 = &acc[B];
                        double* u2 = &acc[2 * B];
#pragma omp simd
                        for (int b = 0; b < B; ++b) {
                            const double ar = c0[b] * c1[b] - s0[b] * s1[b], ai = c0[b] * s1[b] + s0[b] * c1[b];
                            const double br = ar * c2[b] - ai * s2[b], bi = ar * s2[b] + ai * c2[b];
                            const double sv = br * pc - bi * ps;
                            u0[b] += a0 * sv;
                            u1[b] += a1 * sv;
                            u2[b] += a2 * sv;
                        }
                    }
                    for (int d = 0; d < 3; ++d)
                        for (int b = 0; b < nb; ++b) u[d * nd + d0 + b] = acc[d * B + b];
                }
            }
            double usq = 0;
            for (int64_t dof = 0; dof < nd; ++dof)
                for (int d = 0; d < 3; ++d) usq += u[d * nd + dof] * u[d * nd + dof];
            const double urms = std::sqrt(usq / nd);
            const double g = pr.gamma, rho1 = 1.0, p1 = 1.0 / g, a1 = 1.0;  // a = 1 upstream
            const double scale = (urms > 0) ? Mt * a1 / urms : 0;
            const double M2 = Ms * Ms;
            const double rho2 = rho1 * (g + 1) * M2 / ((g - 1) * M2 + 2);
            const double p2 = p1 * (2 * g * M2 - (g - 1)) / (g + 1);
            const double ushock = Ms * a1 * (1 - rho1 / rho2);  // post-shock speed in the lab frame
            for (int64_t dof = 0; dof < nd; ++dof) {
                const bool behind = C.dof_xyz[dof] < xs;
                double vel[3] = {scale * u[dof], scale * u[nd + dof], scale * u[2 * nd + dof]};
                if (behind) vel[0] += ushock;
                double s[5];
                prim_to_cons(g, behind ? rho2 : rho1, vel, behind ? p2 : p1, s);
                setU(dof, s);
            }
        } else if (ic == "from archive restart") {
            // ICs::FromArchiveRestart (IBCs/from_archive_restart.cc:23-73): the state of an archive
            // written for this mesh and degree (this build's own archive format, output.h); the
            // start time and output counter come from the time integration settings, as there
            read_archive(path(prm.get("IC/file name")), C.degree, C.n_cells, nd, C.U0.data(), nullptr, nullptr, nullptr);
        } else {
            throw std::runtime_error("Invalid IC type '" + ic + "'");
        }
        // seeded perturbations of the configs
        const std::string nv = prm.get("IC/noise/variable");
        const double amp = prm.get_double("IC/noise/amplitude");
        if (nv != "none" && amp != 0) {
            std::mt19937_64 rng(static_cast<uint64_t>(prm.get_integer("IC/noise/seed")));
            std::uniform_real_distribution<double> U(-1.0, 1.0);
            for (int64_t dof = 0; dof < nd; ++dof) {
                const double r = U(rng);
                double s[5];
                for (int v = 0; v < 5; ++v) s[v] = C.U0[v * nd + dof];
                const double rho = s[0], vel[3] = {s[1] / rho, s[2] / rho, s[3] / rho};
                const double p = (pr.gamma - 1) * (s[4] - 0.5 * (s[1] * s[1] + s[2] * s[2] + s[3] * s[3]) / rho);
                // additive density noise at fixed velocity and pressure
                if (nv == "rho") {
                    prim_to_cons(pr.gamma, rho + amp * r, vel, p, s);
                } else if (nv == "pre-shock rho") {
                    if (std::fabs(vel[0]) + std::fabs(vel[1]) + std::fabs(vel[2]) == 0)
                        prim_to_cons(pr.gamma, rho + amp * r, vel, p, s);
                } else if (nv == "velocity") {
                    const double r2 = U(rng), r3 = U(rng);
                    const double sp = std::sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
                    const double v2[3] = {vel[0] + amp * sp * r, vel[1] + amp * sp * r2, vel[2] + amp * sp * r3};
                    prim_to_cons(pr.gamma, rho, v2, p, s);
                } else {
                    throw std::runtime_error("IC/noise/variable must be none|rho|pre-shock rho|velocity");
                }
                for (int v = 0; v < 5; ++v) C.U0[v * nd + dof] = s[v];
            }
        }
        // IC::assert_positivity
        for (int64_t dof = 0; dof < nd; ++dof) {
            const double rho = C.U0[dof];
            double ke = 0;
            for (int d = 1; d <= 3; ++d) ke += C.U0[d * nd + dof] * C.U0[d * nd + dof];
            const double e = (C.U0[4 * nd + dof] - 0.5 * ke / rho) / rho;
            if (!(rho > 0) || !(e > 0)) throw std::runtime_error("initial condition is not positive at dof " + std::to_string(dof));
        }
    }
    charge(3);
    C.prm_echo = prm.print_parameters();
    C.finalize_pointers();
    return cs;
}

}  // namespace plens
