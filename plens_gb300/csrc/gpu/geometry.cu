// geometry.cu -- plens_gpu_setup_geometry (include/plens_gpu.h): the metric terms of
// calc_metric_terms / MetricTerms<3>::reinit (dgsem/plens.cc:1646-1682,
// dgsem/metric_terms.cc:67-142) and the face-dof matching of form_neighbor_face_matchings
// (dgsem/plens.cc:1574-1627) with the face normals of calc_surf_flux (dgsem/plens.cc:1751-1756,
// 1797), on the GPU.
//
// Every product, sum, quotient and square root is an explicitly rounded FP64 intrinsic in the
// host setup's order (plens_gb300/csrc/host/setup.cpp, host_setup_geometry), so the results are
// the host's bits whatever the compiler would contract. FP64 is a thin pipe on GB300, but the
// setup is a one-off ~50 FLOP per support point and node: 16.8 M nodes x 8 support points (the
// 64^3-cell box at N=3) take a few ms, against seconds on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "plens_gpu.h"

namespace {

constexpr int kMaxSupport = 8;  // mapping degree <= 7
constexpr int kMaxPoints = 8;   // rule points per direction (fe degree <= 7)
constexpr unsigned long long kNone = ~0ull;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// face-local dof -> cell-local dof (dgsem/face_dof_info.h:92-150); faces 2/3 run x fastest, then z
__device__ __forceinline__ int face_to_cell_dof(int P, int face, int q)
{
    const int a = q % P, b = q / P;
    switch (face) {
    case 0: return P * q;
    case 1: return (P - 1) + P * q;
    case 2: return a + P * P * b;
    case 3: return a + P * (P - 1) + P * P * b;
    case 4: return q;
    default: return q + P * P * (P - 1);
    }
}

// The node whose normal FEFaceValues::normal_vector(q) returns for face dof q: on faces 2/3 the
// face quadrature runs z fastest while the face dofs run x fastest, and dgsem/plens.cc:1790-1797
// uses one index for both.
__device__ __forceinline__ int normal_node_of_face_dof(int P, int face, int q)
{
    if (face == 2 || face == 3) return face_to_cell_dof(P, face, (q % P) * P + (q / P));
    return face_to_cell_dof(P, face, q);
}

// One thread per node of the rule: x = sum_s X_s L_s(xi), J = sum_s X_s (grad L_s)^T, then det J,
// J^-1 by cofactors and Ja^d = a_{d+1} x a_{d+2} with a_d the columns of J.
__global__ void __launch_bounds__(256) k_mapping(int np, int ns, int64_t nc, const double* __restrict__ support,
                                                 const double* __restrict__ basis, const double* __restrict__ dbasis,
                                                 double* __restrict__ xyz, double* __restrict__ detJ,
                                                 double* __restrict__ Ja, double* __restrict__ Jinv,
                                                 unsigned long long* __restrict__ bad_cell)
{
    __shared__ double s_b[kMaxPoints * kMaxSupport], s_db[kMaxPoints * kMaxSupport];
    for (int i = threadIdx.x; i < np * ns; i += blockDim.x) {
        s_b[i] = basis[i];
        s_db[i] = dbasis[i];
    }
    __syncthreads();
    const int np2 = np * np, np3 = np2 * np, ns3 = ns * ns * ns;
    const int64_t nn = nc * np3;
    for (int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; node < nn;
         node += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = node / np3;
        const int l = (int)(node - c * np3);
        const int t0 = l % np, t1 = (l / np) % np, t2 = l / np2;
        const double* X0 = support + c * ns3 * 3;
        double x[3] = {0, 0, 0}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int k = 0; k < ns; ++k)
            for (int j = 0; j < ns; ++j)
                for (int i = 0; i < ns; ++i) {
                    const double* X = X0 + (i + ns * (j + ns * k)) * 3;
                    const double li = s_b[t0 * ns + i], lj = s_b[t1 * ns + j], lk = s_b[t2 * ns + k];
                    const double g[3] = {mul(mul(s_db[t0 * ns + i], lj), lk), mul(mul(li, s_db[t1 * ns + j]), lk),
                                         mul(mul(li, lj), s_db[t2 * ns + k])};
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const double Xd = __ldg(X + d);
                        x[d] = add(x[d], mul(mul(mul(Xd, li), lj), lk));
#pragma unroll
                        for (int e = 0; e < 3; ++e) J[d][e] = add(J[d][e], mul(Xd, g[e]));
                    }
                }
        if (xyz)
#pragma unroll
            for (int d = 0; d < 3; ++d) xyz[d * nn + node] = x[d];
        const double m0 = sub(mul(J[1][1], J[2][2]), mul(J[1][2], J[2][1]));
        const double m1 = sub(mul(J[1][0], J[2][2]), mul(J[1][2], J[2][0]));
        const double m2 = sub(mul(J[1][0], J[2][1]), mul(J[1][1], J[2][0]));
        const double det = add(sub(mul(J[0][0], m0), mul(J[0][1], m1)), mul(J[0][2], m2));
        if (!(det > 0)) atomicMin(bad_cell, (unsigned long long)c);
        if (detJ) detJ[node] = det;
        if (Jinv) {
            const double inv[9] = {
                dvd(sub(mul(J[1][1], J[2][2]), mul(J[1][2], J[2][1])), det),
                dvd(sub(mul(J[0][2], J[2][1]), mul(J[0][1], J[2][2])), det),
                dvd(sub(mul(J[0][1], J[1][2]), mul(J[0][2], J[1][1])), det),
                dvd(sub(mul(J[1][2], J[2][0]), mul(J[1][0], J[2][2])), det),
                dvd(sub(mul(J[0][0], J[2][2]), mul(J[0][2], J[2][0])), det),
                dvd(sub(mul(J[0][2], J[1][0]), mul(J[0][0], J[1][2])), det),
                dvd(sub(mul(J[1][0], J[2][1]), mul(J[1][1], J[2][0])), det),
                dvd(sub(mul(J[0][1], J[2][0]), mul(J[0][0], J[2][1])), det),
                dvd(sub(mul(J[0][0], J[1][1]), mul(J[0][1], J[1][0])), det)};
#pragma unroll
            for (int r = 0; r < 9; ++r) Jinv[r * nn + node] = inv[r];
        }
        if (Ja)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
                const double a1[3] = {J[0][d1], J[1][d1], J[2][d1]};
                const double a2[3] = {J[0][d2], J[1][d2], J[2][d2]};
                Ja[(d * 3 + 0) * nn + node] = sub(mul(a1[1], a2[2]), mul(a1[2], a2[1]));
                Ja[(d * 3 + 1) * nn + node] = sub(mul(a1[2], a2[0]), mul(a1[0], a2[2]));
                Ja[(d * 3 + 2) * nn + node] = sub(mul(a1[0], a2[1]), mul(a1[1], a2[0]));
            }
    }
}

// One thread per face dof of a face task: the matching face dof of the other side (the first whose
// node lies within the benchmark's tolerance, the periodic direction left out), the unit outward normal
// and the location.
__global__ void __launch_bounds__(256) k_face_dofs(int P, int64_t nd, int64_t nt, const double* __restrict__ xyz,
                                                   const double* __restrict__ Ja, const int32_t* __restrict__ ft_cell,
                                                   const int32_t* __restrict__ ft_face,
                                                   const int32_t* __restrict__ ft_nbr_cell,
                                                   const int32_t* __restrict__ ft_nbr_face,
                                                   const int32_t* __restrict__ ft_skip_dir,
                                                   const double* __restrict__ ft_tol, int32_t* __restrict__ nbr_fdof,
                                                   double* __restrict__ normal, double* __restrict__ fxyz,
                                                   unsigned long long* __restrict__ unmatched,
                                                   unsigned long long* __restrict__ misoriented)
{
    const int P2 = P * P, P3 = P2 * P;
    const int64_t n = nt * P2;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx / P2;
        const int q = (int)(idx - t * P2);
        const int64_t c = ft_cell[t], oc = ft_nbr_cell[t];
        const int f = ft_face[t];
        const int64_t own = c * P3 + face_to_cell_dof(P, f, q);
        int match = (oc < 0) ? q : -1;
        if (oc >= 0) {
            const int of = ft_nbr_face[t], pdir = ft_skip_dir[t];
            const double tol = ft_tol[t];
            for (int q2 = 0; q2 < P2 && match < 0; ++q2) {
                const int64_t other = oc * P3 + face_to_cell_dof(P, of, q2);
                double s2 = 0;
                for (int d = 0; d < 3; ++d) {
                    if (d == pdir) continue;
                    const double df = sub(xyz[d * nd + own], xyz[d * nd + other]);
                    s2 = add(s2, mul(df, df));
                }
                if (__dsqrt_rn(s2) < tol) match = q2;
            }
            if (match < 0) atomicMin(unmatched, (unsigned long long)idx);
            else if (pdir >= 0 && match != q) atomicMin(misoriented, (unsigned long long)idx);
        }
        nbr_fdof[idx] = match;
        const int64_t ln = c * P3 + normal_node_of_face_dof(P, f, q);
        const int dir = f / 2;
        const double sgn = (f % 2 == 0) ? -1.0 : 1.0;
        double nv[3], nn = 0;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            nv[e] = Ja[(dir * 3 + e) * nd + ln];
            nn = add(nn, mul(nv[e], nv[e]));
        }
        nn = __dsqrt_rn(nn);
#pragma unroll
        for (int e = 0; e < 3; ++e) normal[idx * 3 + e] = dvd(mul(sgn, nv[e]), nn);
#pragma unroll
        for (int e = 0; e < 3; ++e) fxyz[idx * 3 + e] = xyz[e * nd + own];
    }
}

// Device buffers of one job, freed on every return path.
struct Buffers {
    std::vector<void*> ptrs;
    ~Buffers()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    T* alloc(size_t n)
    {
        void* p = nullptr;
        if (n == 0) n = 1;
        if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

unsigned grid_for(int64_t n, int block)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + block - 1) / block;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 16));
}

}  // namespace

extern "C" int plens_gpu_setup_geometry(plens_geometry_job* j)
{
    if (!j || j->n_points < 1 || j->n_points > kMaxPoints || j->n_support < 2 || j->n_support > kMaxSupport ||
        j->n_cells <= 0 || !j->support || !j->basis || !j->dbasis || j->n_face_tasks < 0)
        return PLENS_GPU_E_INVALID;
    const int np = j->n_points, ns = j->n_support, np3 = np * np * np, ns3 = ns * ns * ns;
    const int64_t nc = j->n_cells, nn = nc * np3, nt = j->n_face_tasks, P2 = (int64_t)np * np;
    if (nt > 0 && (!j->xyz || !j->Ja || !j->ft_cell || !j->ft_face || !j->ft_nbr_cell || !j->ft_nbr_face ||
                   !j->ft_skip_dir || !j->ft_tol || !j->ft_nbr_fdof || !j->ft_normal || !j->ft_xyz))
        return PLENS_GPU_E_INVALID;
    j->first_bad_cell = j->first_unmatched = j->first_misoriented = -1;

    Buffers b;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return PLENS_GPU_E_CUDA;
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    // xyz and Ja are needed on the device by the face kernel even when the caller wants neither
    const bool want_xyz = j->xyz || nt > 0, want_ja = j->Ja || nt > 0;
    double* d_sup = b.alloc<double>((size_t)nc * ns3 * 3);
    double* d_tab = b.alloc<double>(2 * (size_t)np * ns);
    double* d_xyz = want_xyz ? b.alloc<double>(3 * (size_t)nn) : nullptr;
    double* d_det = j->detJ ? b.alloc<double>((size_t)nn) : nullptr;
    double* d_ja = want_ja ? b.alloc<double>(9 * (size_t)nn) : nullptr;
    double* d_jinv = j->Jinv ? b.alloc<double>(9 * (size_t)nn) : nullptr;
    unsigned long long* d_flags = b.alloc<unsigned long long>(3);
    if (!d_sup || !d_tab || (want_xyz && !d_xyz) || (j->detJ && !d_det) || (want_ja && !d_ja) ||
        (j->Jinv && !d_jinv) || !d_flags)
        return PLENS_GPU_E_CUDA;
    const unsigned long long none[3] = {kNone, kNone, kNone};
    bool ok = cudaMemcpyAsync(d_sup, j->support, sizeof(double) * nc * ns3 * 3, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(d_tab, j->basis, sizeof(double) * np * ns, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(d_tab + np * ns, j->dbasis, sizeof(double) * np * ns, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(d_flags, none, sizeof(none), cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (!ok) return PLENS_GPU_E_CUDA;
    k_mapping<<<grid_for(nn, 256), 256, 0, st>>>(np, ns, nc, d_sup, d_tab, d_tab + np * ns, d_xyz, d_det, d_ja,
                                                 d_jinv, d_flags);
    if (cudaGetLastError() != cudaSuccess) return PLENS_GPU_E_CUDA;

    if (nt > 0) {
        int32_t* d_i32 = b.alloc<int32_t>(5 * (size_t)nt + (size_t)nt * P2);
        double* d_tol = b.alloc<double>((size_t)nt);
        double* d_norm = b.alloc<double>((size_t)nt * P2 * 3);
        double* d_fxyz = b.alloc<double>((size_t)nt * P2 * 3);
        if (!d_i32 || !d_tol || !d_norm || !d_fxyz) return PLENS_GPU_E_CUDA;
        const int32_t* src[5] = {j->ft_cell, j->ft_face, j->ft_nbr_cell, j->ft_nbr_face, j->ft_skip_dir};
        for (int a = 0; a < 5; ++a)
            ok = ok && cudaMemcpyAsync(d_i32 + a * nt, src[a], sizeof(int32_t) * nt, cudaMemcpyHostToDevice, st) == cudaSuccess;
        ok = ok && cudaMemcpyAsync(d_tol, j->ft_tol, sizeof(double) * nt, cudaMemcpyHostToDevice, st) == cudaSuccess;
        if (!ok) return PLENS_GPU_E_CUDA;
        int32_t* d_match = d_i32 + 5 * nt;
        k_face_dofs<<<grid_for(nt * P2, 256), 256, 0, st>>>(np, nn, nt, d_xyz, d_ja, d_i32, d_i32 + nt, d_i32 + 2 * nt,
                                                           d_i32 + 3 * nt, d_i32 + 4 * nt, d_tol, d_match, d_norm,
                                                           d_fxyz, d_flags + 1, d_flags + 2);
        if (cudaGetLastError() != cudaSuccess) return PLENS_GPU_E_CUDA;
        ok = cudaMemcpyAsync(j->ft_nbr_fdof, d_match, sizeof(int32_t) * nt * P2, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(j->ft_normal, d_norm, sizeof(double) * nt * P2 * 3, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(j->ft_xyz, d_fxyz, sizeof(double) * nt * P2 * 3, cudaMemcpyDeviceToHost, st) == cudaSuccess;
        if (!ok) return PLENS_GPU_E_CUDA;
    }
    unsigned long long flags[3];
    ok = (!j->xyz || cudaMemcpyAsync(j->xyz, d_xyz, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, st) == cudaSuccess) &&
         (!j->detJ || cudaMemcpyAsync(j->detJ, d_det, sizeof(double) * nn, cudaMemcpyDeviceToHost, st) == cudaSuccess) &&
         (!j->Ja || cudaMemcpyAsync(j->Ja, d_ja, sizeof(double) * 9 * nn, cudaMemcpyDeviceToHost, st) == cudaSuccess) &&
         (!j->Jinv || cudaMemcpyAsync(j->Jinv, d_jinv, sizeof(double) * 9 * nn, cudaMemcpyDeviceToHost, st) == cudaSuccess) &&
         cudaMemcpyAsync(flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) return PLENS_GPU_E_CUDA;
    j->first_bad_cell = flags[0] == kNone ? -1 : (int64_t)flags[0];
    j->first_unmatched = flags[1] == kNone ? -1 : (int64_t)flags[1];
    j->first_misoriented = flags[2] == kNone ? -1 : (int64_t)flags[2];
    return PLENS_GPU_OK;
}
