// plens_gpu.cu -- the C ABI of include/plens_gpu.h: context lifecycle, device buffers and the
// stage orchestration of PLENS::update / update_rk4 / update_rk3 / calc_rhs
// (dgsem/plens.cc:3688-3779, 4334-4518) on one CUDA stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "diagnostics.cuh"
#include "launch.cuh"
#include "mlp.cuh"
#include "plens_gpu.h"

namespace plens_gpu {
LaunchTable table_fp64_2(); LaunchTable table_fp64_3(); LaunchTable table_fp64_4();
LaunchTable table_fp64_5(); LaunchTable table_fp64_6();
LaunchTable table_mixed_2(); LaunchTable table_mixed_3(); LaunchTable table_mixed_4();
LaunchTable table_mixed_5(); LaunchTable table_mixed_6();

static LaunchTable pick_table(int P, bool mixed)
{
    switch (P) {
    case 2: return mixed ? table_mixed_2() : table_fp64_2();
    case 3: return mixed ? table_mixed_3() : table_fp64_3();
    case 4: return mixed ? table_mixed_4() : table_fp64_4();
    case 5: return mixed ? table_mixed_5() : table_fp64_5();
    case 6: return mixed ? table_mixed_6() : table_fp64_6();
    default: return LaunchTable{};
    }
}

// ------------------------------------------------------------------- 1D operators (host)
static void gll(int n, std::vector<double>& x01, std::vector<double>& w01)
{
    const int N = n - 1;
    std::vector<long double> x(n);
    for (int i = 0; i < n; ++i) x[i] = std::cos(M_PI * (long double)i / N);
    for (int it = 0; it < 200; ++it) {
        long double diff = 0;
        for (int i = 0; i < n; ++i) {
            long double a = 1, b = x[i];
            for (int k = 2; k <= N; ++k) { const long double c = ((2 * k - 1) * x[i] * b - (k - 1) * a) / k; a = b; b = c; }
            if (N == 1) a = 1;
            const long double xn = x[i] - (x[i] * b - a) / (n * b);
            diff = std::max(diff, std::fabs(xn - x[i]));
            x[i] = xn;
        }
        if (diff < 1e-19L) break;
    }
    x01.assign(n, 0);
    w01.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        long double a = 1, b = x[i];
        for (int k = 2; k <= N; ++k) { const long double c = ((2 * k - 1) * x[i] * b - (k - 1) * a) / k; a = b; b = c; }
        x01[n - 1 - i] = (double)((x[i] + 1) / 2);
        w01[n - 1 - i] = (double)(1.0L / (N * n * b * b));
    }
    x01[0] = 0;
    x01[n - 1] = 1;
}

static double legendre01(int k, double x)  // orthonormal Legendre polynomial on [0,1]
{
    if (k == 0) return 1.0;
    const double t = 2 * x - 1;
    double a = 1, b = t;
    for (int j = 2; j <= k; ++j) { const double c = ((2 * j - 1) * t * b - (j - 1) * a) / j; a = b; b = c; }
    return std::sqrt(2.0 * k + 1) * b;
}

static Ops make_ops(int P)
{
    Ops o;
    std::memset(&o, 0, sizeof(o));
    std::vector<double> xi, w;
    gll(P, xi, w);
    for (int i = 0; i < P; ++i) o.w[i] = w[i];
    for (int i = 0; i < P; ++i)
        for (int j = 0; j < P; ++j) {
            double s = 0;
            for (int k = 0; k < P; ++k) {
                if (k == j) continue;
                double t = 1.0 / (xi[j] - xi[k]);
                for (int m = 0; m < P; ++m)
                    if (m != j && m != k) t *= (xi[i] - xi[m]) / (xi[j] - xi[m]);
                s += t;
            }
            o.D[i * P + j] = s;
            o.Q[i * P + j] = w[i] * s;
        }
    // Gauss rule with P points on [0,1]
    std::vector<double> gx(P), gw(P);
    for (int i = 0; i < P; ++i) {
        long double x = std::cos(M_PI * (i + 0.75L) / (P + 0.5L)), dp = 0;
        for (int it = 0; it < 100; ++it) {
            long double a = 1, b = x;
            for (int k = 2; k <= P; ++k) { const long double c = ((2 * k - 1) * x * b - (k - 1) * a) / k; a = b; b = c; }
            dp = P * (x * b - a) / (x * x - 1);
            const long double dx = b / dp;
            x -= dx;
            if (std::fabs(dx) < 1e-20L) break;
        }
        gx[P - 1 - i] = (double)((x + 1) / 2);
        gw[P - 1 - i] = (double)(1.0L / ((1 - x * x) * dp * dp));
    }
    for (int a = 0; a < P; ++a)
        for (int i = 0; i < P; ++i) {
            double s = 0;
            for (int g = 0; g < P; ++g) {
                double l = 1;
                for (int m = 0; m < P; ++m)
                    if (m != i) l *= (gx[g] - xi[m]) / (xi[i] - xi[m]);
                s += gw[g] * legendre01(a, gx[g]) * l;
            }
            o.C1[a * P + i] = s;
        }
    for (int i = 0; i < P; ++i) o.fw[i] = (float)o.w[i];
    for (int i = 0; i < P * P; ++i) {
        o.fD[i] = (float)o.D[i];
        o.fQ[i] = (float)o.Q[i];
        o.fC1[i] = (float)o.C1[i];
    }
    o.tv[0] = 0.0;
    if (P > 1) o.tv[1] = std::fabs(legendre01(1, 1) - legendre01(1, 0));
    for (int ip = 2; ip < P; ++ip) {
        std::vector<double> qx, qw;
        gll(ip + 1, qx, qw);
        double tv = 0;
        for (int k = 0; k < ip; ++k) tv += std::fabs(legendre01(ip, qx[k + 1]) - legendre01(ip, qx[k]));
        o.tv[ip] = tv;
    }
    for (int i = 0; i < P; ++i) o.ftv[i] = (float)o.tv[i];
    return o;
}

}  // namespace plens_gpu

using namespace plens_gpu;

struct plens_ctx {
    int P = 0, N = 0;
    int64_t nc = 0, nd = 0, ntask = 0, nslot = 0;
    bool viscous = false, mixed = false, learned = false;
    bool reg64 = false;  // MIXED form: FP64 RK registers, metric terms read in FP64
    // mixed forms at N = 3: the modal indicator's change of basis on the tensor cores (the B
    // operand, made at creation) while indicator_tc is set (the default with the modal sensor)
    float* cbm_tc = nullptr;
    bool indicator_tc = false;
    plens_params prm{};
    Dev dv{};
    Ops ops{};
    GasP gas{};
    BlendP bp{};
    LaunchTable tab{};
    double N15 = 1;
    cudaStream_t stream = nullptr;
    // the troubled-cell indicator (blender or learned sensor, then the smoothing) runs on a side
    // stream, forked from and joined back into `stream` within each RHS: it overlaps the face
    // kernels, which do not read alpha unless the surface flux blends with it
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // mixed forms with the compacted troubled-cell list: the interior subcell sums of the listed
    // cells follow alpha and the list on the side stream; the volume kernel joins them
    cudaEvent_t ev_join_lo = nullptr;
    // the start of a step (stable time step, rho E and state snapshots) runs on a third stream
    // beside stage 1's indicator and face kernels; stage 1's volume kernel, the first to need dt
    // or to write the state, joins it
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_step_fork = nullptr, ev_step_join = nullptr;
    bool step_join_pending = false;
    int64_t launches = 0;
    std::string err = "no error";
    std::vector<void*> allocs;
    double* R[3] = {nullptr, nullptr, nullptr};
    double* Rout = nullptr;
    Scalars* sc = nullptr;
    // page-locked, device-mapped mirror of the device scalars (k_scalars_out writes it)
    Scalars* sc_host = nullptr;
    Scalars* sc_mirror = nullptr;  // its device address
    MlpDevice mlp{};
    int64_t bad_dof_host = -1;
    // volume-kernel timing
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
    size_t ev_used = 0;
    double vol_ms = 0;
    int64_t vol_n = 0;
    // one RK step captured as a CUDA graph and replayed (two variants with the learned sensor:
    // without and with the judge); rebuilt when the end time changes
    cudaGraphExec_t step_graph[2] = {nullptr, nullptr};
    int64_t step_graph_launches[2] = {0, 0};
    double step_graph_end = 0;
    bool use_graphs = true;
    // asynchronous snapshot: device copy on the compute stream, device -> pinned host copy on a
    // second stream while later steps run
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t snap_ready = nullptr, snap_done = nullptr;
    unsigned char* snap_dev = nullptr;
    unsigned char* snap_host = nullptr;
    size_t snap_bytes = 0;
    bool snap_pending = false;
    // sequences of states (plens_gpu_advance_states): the next member's state copied in on one
    // stream, the last member's state copied out on another, each through a device buffer of its
    // own; made on the first call
    cudaStream_t seq_in = nullptr, seq_out = nullptr;
    cudaEvent_t seq_in_ready = nullptr, seq_in_free = nullptr, seq_out_ready = nullptr, seq_out_free = nullptr;
    double *seq_in_buf = nullptr, *seq_out_buf = nullptr;
    // each member's outcome, in page-locked, device-mapped host memory (grown as needed)
    MemberStatus* seq_status_host = nullptr;
    MemberStatus* seq_status_dev = nullptr;
    int64_t seq_status_cap = 0;
    // error norms of the output steps: rho E of the previous step's start, the quadrature data,
    // per-cell and total sums
    double* rhoE_old = nullptr;
    const double *q_wJ = nullptr, *q_xyz = nullptr;
    double *err_cell = nullptr, *err_sum = nullptr;
    GaussInterp gi{};
};

namespace {

int fail(plens_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

int cuda_fail(plens_ctx* c, cudaError_t e, const char* what)
{
    return fail(c, PLENS_GPU_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                         \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
    } while (0)

template <class T>
int dalloc(plens_ctx* c, T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
    c->allocs.push_back(*p);
    return 0;
}

template <class T>
int dupload(plens_ctx* c, const T** dst, const T* src, size_t n)
{
    T* p = nullptr;
    if (int r = dalloc(c, &p, n)) return r;
    if (src && n) {
        cudaError_t e = cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpy H2D");
    }
    *dst = p;
    return 0;
}

int check_launch(plens_ctx* c, const char* what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, what);
    return 0;
}

// The device address of a host buffer that kernels may read and write directly: page-locked and
// mapped memory (cudaHostAlloc, cudaHostRegister; torch's pinned tensors), whose attributes name a
// device pointer. Null for anything else (pageable memory, device memory, errors), which then
// goes through the copy engines.
void* mapped_device_ptr(const void* host)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();  // clear the error of an unknown pointer
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost) ? a.devicePointer : nullptr;
}

// mixed form: the FP32 image of the state after U was written outside the update kernels
int refresh_image(plens_ctx* c)
{
    if (!c->dv.Uf) return 0;
    k_state_image<<<(unsigned)std::min<int64_t>((5 * c->nd + 255) / 256, 152 * 16), 256, 0, c->stream>>>(c->dv);
    c->launches += 1;
    return check_launch(c, "state image");
}

// One RHS of the current stage: calc_rhs without the final store (dgsem/plens.cc:3688-3779).
// The volume kernel of `sa` blends and either stores or advances the registers.
int launch_rhs(plens_ctx* c, const StageArgs& sa)
{
    cudaStream_t st = c->stream;
    // fork: the indicator chain on the side stream (it reads the state and writes only alpha,
    // alpha_d, the troubled-cell list and the positivity status)
    cudaError_t e = cudaEventRecord(c->ev_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_fork, 0);
    if (e != cudaSuccess) return cuda_fail(c, e, "indicator fork");
    if (c->learned) {
        c->launches += mlp_sensor_launch(c->mlp, c->dv, c->ops, c->gas, c->bp, c->P, c->side);
    } else {
        if (c->indicator_tc) c->launches += c->tab.blender_tc(c->dv, c->ops, c->gas, c->bp, c->cbm_tc, c->side);
        else c->launches += c->tab.blender(c->dv, c->ops, c->gas, c->bp, c->side);
        k_alpha_smooth<<<(unsigned)((c->nc + kSmoothThreads - 1) / kSmoothThreads), kSmoothThreads, 0, c->side>>>(c->dv, c->bp);
        ++c->launches;
    }
    if (c->dv.lo_blk && !c->dv.lo_decode) {  // the list, where the subcell kernel does not decode it
        k_lo_list<<<(unsigned)((c->nc + kSmoothThreads - 1) / kSmoothThreads), kSmoothThreads, 0, c->side>>>(c->dv);
        ++c->launches;
    }
    e = cudaEventRecord(c->ev_join, c->side);
    if (e != cudaSuccess) return cuda_fail(c, e, "indicator join");
    if (c->dv.lo_blk) {
        // the interior subcell sums of the listed troubled cells (need alpha and the list only;
        // the volume kernel adds their cell-face terms), still beside the face kernels
        c->launches += c->tab.subcell(c->dv, c->ops, c->gas, c->side);
        e = cudaEventRecord(c->ev_join_lo, c->side);
        if (e != cudaSuccess) return cuda_fail(c, e, "subcell join");
    }
    if (c->viscous) {
        c->launches += c->tab.surface(1, c->dv, c->gas, c->dv.sf, st);
        c->launches += c->tab.aux(c->dv, c->ops, c->gas, st);
        c->launches += c->tab.surface(3, c->dv, c->gas, c->dv.sf3, st);
    }
    // the alpha-blended surface fluxes wait for alpha; the others run beside the indicator
    const int isf = c->prm.inv_surf_flux;
    const bool blended = isf == PLENS_ISF_CHANDRASHEKHAR || isf == PLENS_ISF_RUSANOV_HLLC ||
                         isf == PLENS_ISF_RUSANOV_AUSM_PLUS_UP;
    if (!blended) c->launches += c->tab.surface(2, c->dv, c->gas, c->dv.sf, st);
    e = cudaStreamWaitEvent(st, c->ev_join, 0);
    if (e == cudaSuccess && c->step_join_pending) e = cudaStreamWaitEvent(st, c->ev_step_join, 0);
    if (e != cudaSuccess) return cuda_fail(c, e, "indicator join");
    c->step_join_pending = false;
    if (blended) c->launches += c->tab.surface(2, c->dv, c->gas, c->dv.sf, st);
    if (c->dv.lo_blk) {
        e = cudaStreamWaitEvent(st, c->ev_join_lo, 0);
        if (e != cudaSuccess) return cuda_fail(c, e, "subcell join");
    }
    if (c->timing) {
        if (c->ev_used == c->ev_pool.size()) {
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            c->ev_pool.emplace_back(a, b);
        }
        cudaEventRecord(c->ev_pool[c->ev_used].first, st);
        c->launches += c->tab.volume(c->viscous, c->dv, c->ops, c->gas, sa, st);
        cudaEventRecord(c->ev_pool[c->ev_used].second, st);
        ++c->ev_used;
    } else {
        c->launches += c->tab.volume(c->viscous, c->dv, c->ops, c->gas, sa, st);
    }
    return check_launch(c, "rhs kernels");
}

int launch_time_step(plens_ctx* c, cudaStream_t st = nullptr)
{
    if (!st) st = c->stream;
    k_courant<<<1, 1, 0, st>>>(c->dv, c->prm.expr_courant);
    c->launches += 1;
    c->launches += c->tab.time_step(c->dv, c->gas, c->N15, c->N, st);
    k_dt_finalize<<<1, 1, 0, st>>>(c->dv);
    c->launches += 1;
    if (c->dv.dt_loc) {
        k_local_dt<<<(unsigned)((c->nc + 255) / 256), 256, 0, st>>>(
            c->dv, c->prm.limit_local_step, c->prm.local_start_time, c->prm.local_nbr_factor,
            c->prm.local_global_factor);
        c->launches += 1;
    }
    return check_launch(c, "time step kernels");
}

// RK4(3)5[3R+]N coefficients of Kennedy, Carpenter & Lewis (2000) as used by the reference
// (dgsem/rk4_stage5_register3.cc:12-36)
const double kB[5] = {314199625218.0 / 7198350928319, 6410344372641.0 / 17000082738695,
                      292278564125.0 / 5593752632744, 5010207514426.0 / 21876007855139,
                      5597675544274.0 / 18784428342765};
const double kAo[5] = {4745337637855.0 / 22386579876409, 6808157035527.0 / 13197844641179,
                       4367509502613.0 / 10454198590847, 1236962429870.0 / 3429868089329,
                       5597675544274.0 / 18784428342765};
const double kAi[4] = {546509042554.0 / 9152262712923, 625707605167.0 / 5316659119056,
                       582400652113.0 / 7078426004906, 5010207514426.0 / 21876007855139};

int launch_step(plens_ctx* c, double end_time, bool judge = true)
{
    cudaStream_t st = c->stream;
    k_step_begin<<<1, 1, 0, st>>>(c->dv, end_time);
    c->launches += 1;
    // fork the start of the step: it reads the state, which nothing writes before stage 1's
    // volume kernel, and writes dt, the snapshots and the clock copy, which nothing reads before it
    cudaError_t e = cudaEventRecord(c->ev_step_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->aux, c->ev_step_fork, 0);
    if (e != cudaSuccess) return cuda_fail(c, e, "step fork");
    if (c->rhoE_old) {
        k_save_rhoE<<<(unsigned)std::min<int64_t>((c->nd + 255) / 256, 152 * 8), 256, 0, c->aux>>>(c->dv, c->rhoE_old);
        c->launches += 1;
    }
    if (c->learned) {
        k_snapshot<<<(unsigned)std::min<int64_t>((5 * c->nd / 2 + 255) / 256, 152 * 16), 256, 0, c->aux>>>(c->dv);
        c->launches += 1;
        if (judge) c->launches += mlp_step_begin(c->mlp, c->dv, c->prm.judge_every, st);
    }
    if (int r = launch_time_step(c, c->aux)) return r;
    e = cudaEventRecord(c->ev_step_join, c->aux);
    if (e != cudaSuccess) return cuda_fail(c, e, "step join");
    c->step_join_pending = true;
    if (c->prm.rk_order == 4) {
        // registers rotate: stage s writes dt*R into R[w]; R1 = previous, R0 = previous-previous
        int w = 0, r1 = -1, r0 = -1;
        for (int s = 1; s <= 5; ++s) {
            StageArgs sa{};
            sa.mode = 1;
            sa.stage = s;
            sa.keep = s < 5 ? 1 : 0;  // the last stage's dt*R is read by no later stage
            sa.Rw = c->R[w];
            sa.R1 = (r1 >= 0) ? c->R[r1] : nullptr;
            sa.R0 = (r0 >= 0) ? c->R[r0] : nullptr;
            if (s == 1) {
                sa.c2 = kAo[0];
            } else if (s == 2) {
                sa.c1 = kAi[0] - kAo[0];
                sa.c2 = kAo[1];
            } else {
                sa.c0 = kB[s - 3] - kAi[s - 3];
                sa.c1 = kAi[s - 2] - kAo[s - 2];
                sa.c2 = kAo[s - 1];
            }
            sa.fc0 = (float)sa.c0;
            sa.fc1 = (float)sa.c1;
            sa.fc2 = (float)sa.c2;
            sa.reg64 = c->reg64 ? 1 : 0;
            if (int r = launch_rhs(c, sa)) return r;
            r0 = r1;
            r1 = w;
            w = (w + 1) % 3;
        }
    } else {
        cudaError_t e = cudaMemcpyAsync(c->dv.U0, c->dv.U, sizeof(double) * 5 * c->nd, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(c, e, "U0 copy");
        for (int s = 1; s <= 3; ++s) {
            StageArgs sa{};
            sa.mode = 2;
            sa.stage = s;
            sa.reg64 = c->reg64 ? 1 : 0;
            if (int r = launch_rhs(c, sa)) return r;
        }
    }
    if (c->learned) c->launches += mlp_step_end(c->mlp, c->dv, st);
    k_clock<<<1, 1, 0, st>>>(c->dv);
    c->launches += 1;
    return check_launch(c, "step kernels");
}

// the device scalars as the stream's work so far leaves them (synchronises the stream)
int read_scalars(plens_ctx* c, Scalars* h)
{
    k_scalars_out<<<1, 1, 0, c->stream>>>(c->dv, c->sc_mirror);
    c->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "read scalars");
    *h = *c->sc_host;
    return 0;
}

int sync_and_check(plens_ctx* c)
{
    k_scalars_out<<<1, 1, 0, c->stream>>>(c->dv, c->sc_mirror);
    c->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamSynchronize");
    for (size_t i = 0; i < c->ev_used; ++i) {
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev_pool[i].first, c->ev_pool[i].second);
        c->vol_ms += ms;
        ++c->vol_n;
    }
    c->ev_used = 0;
    const Scalars h = *c->sc_host;
    if (h.err == PLENS_GPU_E_POSITIVITY) {
        c->bad_dof_host = h.bad_dof;
        char buf[160];
        std::snprintf(buf, sizeof(buf), "Positivity assertion failed at dof %lld", h.bad_dof);
        return fail(c, PLENS_GPU_E_POSITIVITY, buf);
    }
    if (h.err) return fail(c, h.err, "device error " + std::to_string(h.err));
    return 0;
}

}  // namespace

extern "C" {

int plens_gpu_create(const plens_mesh_desc* mesh, const plens_params* prm, plens_ctx** out)
{
    if (!out) return PLENS_GPU_E_INVALID;
    *out = nullptr;
    if (!mesh || !prm) return PLENS_GPU_E_INVALID;
    plens_ctx* c = new plens_ctx();
    *out = c;
    if (mesh->degree < 1 || mesh->degree > kMaxP - 1 || mesh->degree != prm->degree)
        return fail(c, PLENS_GPU_E_INVALID, "degree must lie in [1,5] and match the parameters");
    if (mesh->n_cells <= 0 || mesh->n_cells > INT32_MAX) return fail(c, PLENS_GPU_E_INVALID, "bad n_cells");
    if (prm->rk_order != 3 && prm->rk_order != 4) return fail(c, PLENS_GPU_E_INVALID, "RK order must be 3 or 4");
    if (prm->blender_function != 0 && prm->blender_function != 1)
        return fail(c, PLENS_GPU_E_INVALID, "blender function must be Hennemann or linear");
    if (prm->inv_surf_flux < 0 || prm->inv_surf_flux > PLENS_ISF_CHANDRASHEKHAR)
        return fail(c, PLENS_GPU_E_INVALID, "inviscid surface flux scheme not supported on the GPU path");
    if (prm->inv_vol_flux < 0 || prm->inv_vol_flux > PLENS_IVF_ISMAIL_ROE)
        return fail(c, PLENS_GPU_E_INVALID, "bad inviscid volume flux scheme");
    for (int b = 0; b < prm->n_bc; ++b)
        if (prm->bcs[b].type < PLENS_BC_NONE || prm->bcs[b].type > PLENS_BC_ZPG_INFLOW)
            return fail(c, PLENS_GPU_E_INVALID, "bad boundary condition type");
    c->P = mesh->degree + 1;
    c->N = mesh->degree;
    c->nc = mesh->n_cells;
    const int P2 = c->P * c->P, P3 = P2 * c->P;
    c->nd = c->nc * P3;
    c->ntask = mesh->n_face_tasks;
    c->nslot = c->nc * 6 * P2;
    c->prm = *prm;
    c->viscous = !(prm->mu0 < 1e-16);
    if (prm->precision != PLENS_PRECISION_FP64 && prm->precision != PLENS_PRECISION_MIXED &&
        prm->precision != PLENS_PRECISION_MIXED_R32)
        return fail(c, PLENS_GPU_E_INVALID, "bad precision");
    c->mixed = prm->precision != PLENS_PRECISION_FP64;
    c->reg64 = prm->precision == PLENS_PRECISION_MIXED;
    c->learned = prm->sensor == PLENS_SENSOR_LEARNED;
    c->tab = pick_table(c->P, c->mixed);
    if (!c->tab.volume) return fail(c, PLENS_GPU_E_INVALID, "no kernels for this degree");
    c->ops = make_ops(c->P);
    c->N15 = std::pow(c->N, 1.5);
    c->gas = GasP{prm->gamma, prm->R, prm->Pr, prm->mu0, prm->T0, prm->S,
                  prm->const_viscosity, c->viscous ? 0 : 1, prm->inv_surf_flux, prm->inv_vol_flux, prm->plens_2d};
    c->bp.thr = prm->threshold_factor * std::pow(10, -prm->threshold_exp_factor * (std::pow(c->N + 1, 0.25)));
    c->bp.sharp = prm->sharpness_factor;
    c->bp.amin = prm->alpha_min;
    c->bp.amax = prm->alpha_max;
    c->bp.func = prm->blender_function;
    c->bp.var = prm->blender_variable;
    c->bp.expr_wall = prm->expr_wall_blender_limit;
    c->bp.expr_vis = prm->expr_vis_blending_region;
    c->bp.expr_courant = prm->expr_courant;
    c->bp.do_filter = prm->do_filtering;

    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_join_lo, cudaEventDisableTiming));
    CK(cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->ev_step_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_step_join, cudaEventDisableTiming));
    const int64_t nd = c->nd, nc = c->nc, nt = c->ntask;
    Dev& d = c->dv;
    d.nc = nc;
    d.nd = nd;
    d.ntask = nt;
    d.nslot = c->nslot;
    int r = 0;
    if ((r = dupload(c, &d.detJ, mesh->detJ, nd)) || (r = dupload(c, &d.Ja, mesh->Ja, 9 * nd)) ||
        (r = dupload(c, &d.Jinv, mesh->Jinv, 9 * nd)) || (r = dupload(c, &d.h_min, mesh->h_min, nc)) ||
        (r = dupload(c, &d.center, mesh->cell_center, 3 * nc)) || (r = dupload(c, &d.cell_nbr, mesh->cell_nbr, 6 * nc)) ||
        (r = dupload(c, &d.ft_cell, mesh->ft_cell, nt)) || (r = dupload(c, &d.ft_face, mesh->ft_face, nt)) ||
        (r = dupload(c, &d.ft_nbr_cell, mesh->ft_nbr_cell, nt)) || (r = dupload(c, &d.ft_nbr_face, mesh->ft_nbr_face, nt)) ||
        (r = dupload(c, &d.ft_bc, mesh->ft_bc, nt)) || (r = dupload(c, &d.ft_nbr_fdof, mesh->ft_nbr_fdof, nt * P2)) ||
        (r = dupload(c, &d.ft_normal, mesh->ft_normal, nt * P2 * 3)) || (r = dupload(c, &d.ft_xyz, mesh->ft_xyz, nt * P2 * 3)) ||
        (r = dupload(c, &d.bcs, prm->bcs, prm->n_bc)) ||
        (r = dupload(c, &d.expr_code, prm->expr_code, prm->n_expr_insn)) ||
        (r = dupload(c, &d.expr_off, prm->expr_offset, prm->n_expr)) ||
        (r = dupload(c, &d.expr_len, prm->expr_length, prm->n_expr)))
        return r;
    d.n_bc = prm->n_bc;
    d.n_expr = prm->n_expr;
    // per face dof: both sides' dofs and face slots (32-bit: the mesh must have fewer than 2^31
    // dofs and face slots)
    {
        if (nd >= (int64_t)INT32_MAX || c->nslot >= (int64_t)INT32_MAX)
            return fail(c, PLENS_GPU_E_INVALID, "mesh too large for 32-bit face tables");
        const int P = c->P;
        auto fnode = [P, P2](int f, int q) {
            const int N = P - 1;
            switch (f) {
            case 0: return P * q;
            case 1: return N + P * q;
            case 2: return (q % P) + P2 * (q / P);
            case 3: return P * N + (q % P) + P2 * (q / P);
            case 4: return q;
            default: return N * P2 + q;
            }
        };
        const int64_t nfd = nt * P2;
        std::vector<int32_t> own(nfd), nbr(nfd), sown(nfd), snbr(nfd);
        for (int64_t t = 0; t < nt; ++t) {
            const int64_t cc = mesh->ft_cell[t];
            const int f = mesh->ft_face[t], bc = mesh->ft_bc[t];
            const bool periodic = bc >= 0 && bc < prm->n_bc && prm->bcs[bc].type == PLENS_BC_PERIODIC;
            for (int q = 0; q < P2; ++q) {
                const int64_t k = t * P2 + q;
                own[k] = (int32_t)(cc * P3 + fnode(f, q));
                sown[k] = (int32_t)((cc * 6 + f) * P2 + q);
                if (bc < 0 || periodic) {
                    const int64_t nb = mesh->ft_nbr_cell[t];
                    const int fn = mesh->ft_nbr_face[t], qn = mesh->ft_nbr_fdof[k];
                    nbr[k] = (int32_t)(nb * P3 + fnode(fn, qn));
                    snbr[k] = (bc < 0) ? (int32_t)((nb * 6 + fn) * P2 + qn) : -1;
                } else {
                    nbr[k] = -1;
                    snbr[k] = -1;
                }
            }
        }
        if ((r = dupload(c, &d.fd_own, own.data(), nfd)) || (r = dupload(c, &d.fd_nbr, nbr.data(), nfd)) ||
            (r = dupload(c, &d.fs_own, sown.data(), nfd)) || (r = dupload(c, &d.fs_nbr, snbr.data(), nfd)))
            return r;
        if (c->mixed) {
            // periodic pairs merged (owner: the smaller cell*6+face key) unless the scheme blends
            // with alpha (the reference's own-alpha rule for periodic faces then applies per side)
            const int isf = prm->inv_surf_flux;
            const bool merge = isf != PLENS_ISF_CHANDRASHEKHAR && isf != PLENS_ISF_RUSANOV_HLLC &&
                               isf != PLENS_ISF_RUSANOV_AUSM_PLUS_UP;
            std::vector<int4> mdofs;
            std::vector<float4> mgeom;
            for (int64_t t = 0; t < nt; ++t) {
                const int bc = mesh->ft_bc[t];
                const bool periodic = bc >= 0 && bc < prm->n_bc && prm->bcs[bc].type == PLENS_BC_PERIODIC;
                const int64_t key = (int64_t)mesh->ft_cell[t] * 6 + mesh->ft_face[t];
                const int64_t pkey = periodic ? (int64_t)mesh->ft_nbr_cell[t] * 6 + mesh->ft_nbr_face[t] : -1;
                if (periodic && merge && pkey < key) continue;  // the partner's task computes it
                for (int q = 0; q < P2; ++q) {
                    const int64_t k = t * P2 + q;
                    int32_t slot_nb = snbr[k];
                    if (periodic && merge) {
                        const int64_t nb = mesh->ft_nbr_cell[t];
                        const int fn = mesh->ft_nbr_face[t], qn = mesh->ft_nbr_fdof[k];
                        slot_nb = (int32_t)((nb * 6 + fn) * P2 + qn);
                    }
                    mdofs.push_back(make_int4(own[k], nbr[k], sown[k], slot_nb));
                    // round to nearest, as f64_to_f32 on the device
                    const float n0 = (float)mesh->ft_normal[3 * k], n1 = (float)mesh->ft_normal[3 * k + 1],
                                n2 = (float)mesh->ft_normal[3 * k + 2];
                    int32_t kk = (int32_t)k;
                    float kf;
                    std::memcpy(&kf, &kk, sizeof(kf));
                    mgeom.push_back(make_float4(n0, n1, n2, kf));
                }
            }
            d.n_mx = (int64_t)mdofs.size();
            if ((r = dupload(c, &d.mx_dofs, mdofs.data(), mdofs.size())) || (r = dupload(c, &d.mx_geom, mgeom.data(), mgeom.size())))
                return r;
        }
    }
    // wall cells: a boundary face of type uniform temp wall or insulated wall
    // (dgsem/plens.cc:2909-2920)
    {
        std::vector<uint8_t> wall(nc, 0);
        for (int64_t cc = 0; cc < nc; ++cc)
            for (int f = 0; f < 6; ++f) {
                const int b = mesh->cell_face_bc[6 * cc + f];
                if (b >= 0 && b < prm->n_bc &&
                    (prm->bcs[b].type == PLENS_BC_UNIFORM_TEMP_WALL || prm->bcs[b].type == PLENS_BC_INSULATED_WALL))
                    wall[cc] = 1;
            }
        if ((r = dupload(c, &d.cell_wall, wall.data(), nc))) return r;
    }
    if (c->mixed && (r = dalloc(c, &d.Uf, 5 * nd))) return r;
    if (c->reg64) {
        // MIXED form: 1/detJ in FP64, by which the volume kernels scale the FP32 residual sums
        double* invJ = nullptr;
        if ((r = dalloc(c, &invJ, nd))) return r;
        CK(cudaDeviceSynchronize());  // the uploads above ran on the legacy stream
        k_reciprocal<<<(unsigned)std::min<int64_t>((nd + 255) / 256, 152 * 16), 256, 0, c->stream>>>(d.detJ, invJ, nd);
        // The FP32 consumers of the metric terms (the time step's estimate from J^-1; the
        // volume, auxiliary-variable and subcell kernels' FP32 arithmetic on Ja and det J) read
        // the FP32 rounding of the FP64 arrays from images made once: the same values as
        // rounding the FP64 arrays where they are read, half the bytes and no conversions.
        // 1/detJ and the register arithmetic stay FP64.
        float *Jinvf = nullptr, *Jaf = nullptr, *detJf = nullptr;
        if ((r = dalloc(c, &Jinvf, 9 * nd)) || (r = dalloc(c, &Jaf, 9 * nd)) || (r = dalloc(c, &detJf, nd))) return r;
        const unsigned grid = (unsigned)std::min<int64_t>((9 * nd + 255) / 256, 152 * 16);
        k_round_f32<<<grid, 256, 0, c->stream>>>(d.Jinv, Jinvf, 9 * nd);
        k_round_f32<<<grid, 256, 0, c->stream>>>(d.Ja, Jaf, 9 * nd);
        k_round_f32<<<grid, 256, 0, c->stream>>>(d.detJ, detJf, nd);
        c->launches += 4;
        if ((r = check_launch(c, "1/detJ, metric images"))) return r;
        d.invJ = invJ;
        d.Jinvf = Jinvf;
        d.Jaf = Jaf;
        d.detJf = detJf;
    } else if (c->mixed) {
        // MIXED_R32 form: the FP32 rounding of the metric terms, once (every FP32 consumer reads
        // these instead of rounding the FP64 arrays itself: the same values)
        float *detJf = nullptr, *Jaf = nullptr, *Jinvf = nullptr;
        if ((r = dalloc(c, &detJf, nd)) || (r = dalloc(c, &Jaf, 9 * nd)) || (r = dalloc(c, &Jinvf, 9 * nd))) return r;
        // the uploads above ran on the legacy stream, which this non-blocking stream does not
        // wait for (a pageable cudaMemcpy may return before its DMA lands)
        CK(cudaDeviceSynchronize());
        const unsigned grid = (unsigned)std::min<int64_t>((9 * nd + 255) / 256, 152 * 16);
        k_round_f32<<<grid, 256, 0, c->stream>>>(d.detJ, detJf, nd);
        k_round_f32<<<grid, 256, 0, c->stream>>>(d.Ja, Jaf, 9 * nd);
        k_round_f32<<<grid, 256, 0, c->stream>>>(d.Jinv, Jinvf, 9 * nd);
        c->launches += 3;
        if ((r = check_launch(c, "metric images"))) return r;
        d.detJf = detJf;
        d.Jaf = Jaf;
        d.Jinvf = Jinvf;
    }
    if (c->tab.blender_tc) {
        // the B operand of the tensor-core modal indicator (64 x 64 change of basis, TF32 hi/lo)
        std::vector<float> op(2 * 64 * 64 + 64);
        blender_tc_operand(c->ops.C1, op.data());
        if ((r = dalloc(c, &c->cbm_tc, op.size()))) return r;
        CK(cudaMemcpy(c->cbm_tc, op.data(), sizeof(float) * op.size(), cudaMemcpyHostToDevice));
        // the default where it applies: measured faster than the separable CUDA-core transform
        c->indicator_tc = !c->learned;
    }
    if ((r = dalloc(c, &d.U, 5 * nd)) || (r = dalloc(c, &d.alpha_raw, nc)) || (r = dalloc(c, &d.alpha, nc)) ||
        (r = dalloc(c, &d.alpha_d, nc)) || (r = dalloc(c, &d.sf, 5 * c->nslot)) || (r = dalloc(c, &c->sc, 1)) ||
        (r = dalloc(c, &c->Rout, 5 * nd)))
        return r;
    if (prm->do_filtering && (r = dalloc(c, &d.tvstat, 3 * nc))) return r;
    if (prm->rk_order == 4) {
        for (int k = 0; k < 3; ++k)
            if ((r = dalloc(c, &c->R[k], 5 * nd))) return r;
    }
    // step-start state: RK3 needs it; the learned sensor restores it to redo a step with the
    // plain indicator after a positivity failure
    if ((prm->rk_order == 3 || c->learned) && (r = dalloc(c, &d.U0, 5 * nd))) return r;
    if (c->viscous) {
        if ((r = dalloc(c, &d.sf3, 5 * c->nslot)) || (r = dalloc(c, &d.avars, 9 * nd))) return r;
        CK(cudaMemset(d.avars, 0, sizeof(double) * 9 * nd));
    }
    if (prm->calc_ss_error || prm->calc_conv_error) {
        if (!mesh->q_wJ || !mesh->gauss_interp || (prm->calc_conv_error && !mesh->q_xyz) ||
            (prm->calc_conv_error && (prm->expr_conv_exact < 0 || prm->expr_conv_exact >= prm->n_expr)))
            return fail(c, PLENS_GPU_E_INVALID, "error norms requested without their quadrature data or expression");
        if ((r = dupload(c, &c->q_wJ, mesh->q_wJ, nd))) return r;
        if (prm->calc_conv_error && (r = dupload(c, &c->q_xyz, mesh->q_xyz, 3 * nd))) return r;
        if (prm->calc_ss_error) {
            if ((r = dalloc(c, &c->rhoE_old, nd))) return r;
            CK(cudaMemset(c->rhoE_old, 0, sizeof(double) * nd));  // rhoE_old before the first step
        }
        if ((r = dalloc(c, &c->err_cell, 3 * nc)) || (r = dalloc(c, &c->err_sum, 3))) return r;
        for (int i = 0; i < c->P * c->P; ++i) c->gi.g[i] = mesh->gauss_interp[i];
    }
    if (prm->local_stepping) {
        if ((r = dalloc(c, &d.dt_cell, nc)) || (r = dalloc(c, &d.dt_loc, nc))) return r;
        CK(cudaMemset(d.dt_loc, 0, sizeof(double) * nc));
    }
    if (c->mixed && c->tab.uses_lo_list(c->gas)) {
        // the compacted troubled-cell list and the subcell sums of the listed cells
        const int64_t nblk = (nc + kSmoothThreads - 1) / kSmoothThreads;
        if ((r = dalloc(c, &d.lo_list, nc)) || (r = dalloc(c, &d.lo_count, 1)) || (r = dalloc(c, &d.lo_blk, nblk)) ||
            (r = dalloc(c, &d.lo_mask, 4 * nblk)) || (r = dalloc(c, &d.lo_buf, 5 * nd)))
            return r;
        CK(cudaMemset(d.lo_count, 0, sizeof(int32_t)));
        CK(cudaMemset(d.lo_list, 0, sizeof(int32_t) * nc));
        // the subcell kernel finds each list position's cell itself while the smoothing blocks'
        // prefix sums fit 32 KB of its shared memory (up to 1,048,448 cells); larger meshes take
        // k_lo_list first
        d.lo_decode = (nblk + 1 <= kLoDecodeMaxBlocks) ? 1 : 0;
    }
    if (c->learned) {
        if ((r = mlp_create(c->mlp, nc, c->allocs))) return fail(c, PLENS_GPU_E_CUDA, "mlp buffers");
        // degree 3: the fused tensor-core sensor (its change of basis operand), the default there:
        // measured faster than the CUDA-core inference kernel
        c->mlp.cbm = c->cbm_tc;
        c->mlp.use_tc = c->cbm_tc != nullptr;
        c->mlp.tol = prm->judge_alpha_tol;
    }
    d.sc = c->sc;
    CK(cudaHostAlloc(reinterpret_cast<void**>(&c->sc_host), sizeof(Scalars), cudaHostAllocMapped));
    CK(cudaHostGetDevicePointer(reinterpret_cast<void**>(&c->sc_mirror), c->sc_host, 0));
    CK(cudaMemset(d.alpha, 0, sizeof(double) * nc));
    CK(cudaMemset(d.alpha_raw, 0, sizeof(double) * nc));
    CK(cudaMemset(d.alpha_d, 0, sizeof(double) * nc));
    Scalars h{};
    h.time = 0;
    h.bad_dof = INT64_MAX;
    h.dtmin = ord_double_host(1e6);
    CK(cudaMemcpy(c->sc, &h, sizeof(h), cudaMemcpyHostToDevice));
    return 0;
}

int plens_gpu_set_kernel_timing(plens_ctx* c, int enable)
{
    if (!c) return PLENS_GPU_E_INVALID;
    if (int r = sync_and_check(c)) return r;
    c->timing = enable != 0;
    c->vol_ms = 0;
    c->vol_n = 0;
    return 0;
}

int plens_gpu_kernel_timing(plens_ctx* c, double* volume_ms, int64_t* volume_launches)
{
    if (!c) return PLENS_GPU_E_INVALID;
    if (int r = sync_and_check(c)) return r;
    if (volume_ms) *volume_ms = c->vol_ms;
    if (volume_launches) *volume_launches = c->vol_n;
    return 0;
}

int plens_gpu_destroy(plens_ctx* c)
{
    if (!c) return 0;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& pr : c->ev_pool) {
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    for (auto& gx : c->step_graph)
        if (gx) cudaGraphExecDestroy(gx);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    if (c->snap_host) cudaFreeHost(c->snap_host);
    if (c->sc_host) cudaFreeHost(c->sc_host);
    if (c->seq_status_host) cudaFreeHost(c->seq_status_host);
    if (c->snap_dev) cudaFree(c->snap_dev);
    if (c->snap_ready) cudaEventDestroy(c->snap_ready);
    if (c->snap_done) cudaEventDestroy(c->snap_done);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (cudaStream_t s : {c->seq_in, c->seq_out})
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    for (cudaEvent_t e : {c->seq_in_ready, c->seq_in_free, c->seq_out_ready, c->seq_out_free})
        if (e) cudaEventDestroy(e);
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->aux) cudaStreamSynchronize(c->aux);
    for (void* p : c->allocs) cudaFree(p);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_join_lo) cudaEventDestroy(c->ev_join_lo);
    if (c->ev_step_fork) cudaEventDestroy(c->ev_step_fork);
    if (c->ev_step_join) cudaEventDestroy(c->ev_step_join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return 0;
}

__attribute__((visibility("hidden"))) const char* plens_gpu_noalloc_last_error_message();  // noalloc.cu
const char* plens_gpu_last_error(const plens_ctx* c) { return c ? c->err.c_str() : plens_gpu_noalloc_last_error_message(); }
int64_t plens_gpu_kernel_launches(const plens_ctx* c) { return c ? c->launches : 0; }
void* plens_gpu_stream(const plens_ctx* c) { return c ? (void*)c->stream : nullptr; }

int plens_gpu_set_state(plens_ctx* c, const double* U)
{
    if (!c || !U || !c->dv.U) return PLENS_GPU_E_INVALID;
    const int64_t n = 5 * c->nd;
    if (const double* mapped = static_cast<const double*>(mapped_device_ptr(U))) {
        // page-locked host buffer: the SMs read it over the host link and write the state and its
        // FP32 image in one pass (faster than a copy engine, and no second pass for the image)
        k_state_in<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, c->stream>>>(c->dv, mapped);
        c->launches += 1;
        if (int r = check_launch(c, "state in")) return r;
    } else {
        CK(cudaMemcpyAsync(c->dv.U, U, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        if (int r = refresh_image(c)) return r;
    }
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int plens_gpu_get_state(plens_ctx* c, double* U)
{
    if (!c || !U || !c->dv.U) return PLENS_GPU_E_INVALID;
    const int64_t n = 5 * c->nd;
    if (double* mapped = static_cast<double*>(mapped_device_ptr(U))) {
        k_state_out<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, c->stream>>>(c->dv, mapped);
        c->launches += 1;
        if (int r = check_launch(c, "state out")) return r;
    } else {
        CK(cudaMemcpyAsync(U, c->dv.U, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int plens_gpu_set_time(plens_ctx* c, double t, int64_t n_steps)
{
    if (!c || !c->sc) return PLENS_GPU_E_INVALID;
    Scalars h;
    if (int r = read_scalars(c, &h)) return r;
    h.time = t;
    h.n_steps = n_steps;
    h.err = 0;
    h.bad_dof = INT64_MAX;
    CK(cudaMemcpy(c->sc, &h, sizeof(h), cudaMemcpyHostToDevice));
    return 0;
}

int plens_gpu_get_time(plens_ctx* c, double* t, int64_t* n_steps, double* last_dt)
{
    if (!c || !c->sc) return PLENS_GPU_E_INVALID;
    Scalars h;
    if (int r = read_scalars(c, &h)) return r;
    if (t) *t = h.time;
    if (n_steps) *n_steps = h.n_steps;
    if (last_dt) *last_dt = h.dt;
    return 0;
}

int plens_gpu_rhs(plens_ctx* c, double* R_out)
{
    if (!c || !c->dv.U) return PLENS_GPU_E_INVALID;
    if (c->learned && !c->mlp.weights_set) return fail(c, PLENS_GPU_E_INVALID, "learned sensor: weights not set");
    k_step_begin<<<1, 1, 0, c->stream>>>(c->dv, 1e300);
    c->launches += 1;
    if (c->learned) c->launches += mlp_step_begin(c->mlp, c->dv, 1, c->stream);
    StageArgs sa{};
    sa.mode = 0;
    sa.Rout = c->Rout;
    sa.reg64 = c->reg64 ? 1 : 0;
    if (int r = launch_rhs(c, sa)) return r;
    if (int r = sync_and_check(c)) return r;
    if (R_out) CK(cudaMemcpy(R_out, c->Rout, sizeof(double) * 5 * c->nd, cudaMemcpyDeviceToHost));
    return 0;
}

int plens_gpu_time_step(plens_ctx* c, double* dt_out)
{
    if (!c || !c->dv.U) return PLENS_GPU_E_INVALID;
    k_step_begin<<<1, 1, 0, c->stream>>>(c->dv, 1e300);
    c->launches += 1;
    if (int r = launch_time_step(c)) return r;
    if (int r = sync_and_check(c)) return r;
    if (dt_out) *dt_out = c->sc_host->dt_update;  // the mirror sync_and_check read
    return 0;
}

namespace {

// One step through its CUDA graph: the launch sequence of a step is the same every step (the
// kernels read time, dt and the sensor state from device scalars), so it is captured once per
// variant and replayed; the host-side judge schedule of the learned sensor picks the variant.
int graph_step(plens_ctx* c, double end_time)
{
    if (c->step_graph_end != end_time) {
        for (auto& gx : c->step_graph)
            if (gx) {
                cudaGraphExecDestroy(gx);
                gx = nullptr;
            }
        c->step_graph_end = end_time;
    }
    bool judged = false;
    if (c->learned) {
        mlp_step_begin(c->mlp, c->dv, c->prm.judge_every, c->stream);
        judged = c->mlp.judge_this_step;
    }
    const int v = judged ? 1 : 0;
    if (!c->step_graph[v]) {
        cudaGraph_t g = nullptr;
        const int64_t l0 = c->launches;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
        const int r = launch_step(c, end_time, false);
        const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (r) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
        const cudaError_t e2 = cudaGraphInstantiate(&c->step_graph[v], g, 0);
        cudaGraphDestroy(g);
        if (e2 != cudaSuccess) return cuda_fail(c, e2, "cudaGraphInstantiate");
        c->step_graph_launches[v] = c->launches - l0;
        c->launches = l0;
    }
    if (c->learned) c->mlp.judge_this_step = false;
    CK(cudaGraphLaunch(c->step_graph[v], c->stream));
    c->launches += c->step_graph_launches[v];
    return 0;
}

int run_step(plens_ctx* c, double end_time)
{
    // graphs need the launch sequence to be fixed: not while volume-kernel events are recorded
    if (c->use_graphs && !c->timing) return graph_step(c, end_time);
    return launch_step(c, end_time);
}

}  // namespace

int plens_gpu_advance_async(plens_ctx* c, int64_t n_steps, double end_time)
{
    if (!c || !c->dv.U || n_steps < 0) return PLENS_GPU_E_INVALID;
    if (c->learned && !c->mlp.weights_set) return fail(c, PLENS_GPU_E_INVALID, "learned sensor: weights not set");
    for (int64_t s = 0; s < n_steps; ++s)
        if (int r = run_step(c, end_time)) return r;
    return 0;
}

int plens_gpu_synchronize(plens_ctx* c)
{
    if (!c) return PLENS_GPU_E_INVALID;
    return sync_and_check(c);
}

}  // extern "C"

namespace {

// The learned sensor's advance: steps are launched in batches; each step first snapshots its
// start state and clock on the device. A positivity failure deactivates the rest of the batch
// (k_step_begin), and the failed step is redone from its snapshot with the plain modal indicator
// on the whole domain (the fallback lasts until the next judged step). `start`: the clock at the
// call (time and step count) when the caller knows it, which saves reading the device scalars.
int advance_learned(plens_ctx* c, int64_t n_steps, double end_time, const Scalars* start)
{
    constexpr int64_t kBatch = 64;
    int64_t done = 0;
    while (done < n_steps) {
        Scalars h0;
        if (start && done == 0) {
            h0 = *start;
        } else if (int r = read_scalars(c, &h0)) {
            return r;
        }
        if (!(h0.time < end_time)) break;
        const int64_t nb = std::min<int64_t>(kBatch, n_steps - done);
        const int counter0 = c->mlp.step_counter;
        for (int64_t k = 0; k < nb; ++k)
            if (int r = run_step(c, end_time)) return r;
        const int r = sync_and_check(c);
        if (r != PLENS_GPU_E_POSITIVITY) {
            if (r) return r;
            done += nb;
            continue;
        }
        Scalars h = *c->sc_host;  // the mirror sync_and_check read
        if (h.sensor_fallback) return r;  // the plain indicator was in use: report it
        const int64_t ok_steps = h.n_steps0 - h0.n_steps;  // steps of the batch before the failed one
        CK(cudaMemcpyAsync(c->dv.U, c->dv.U0, sizeof(double) * 5 * c->nd, cudaMemcpyDeviceToDevice, c->stream));
        if (int r2 = refresh_image(c)) return r2;
        h.time = h.time0;
        h.n_steps = h.n_steps0;
        h.sensor_fallback = 1;
        h.fallbacks += c->nc;  // every cell handed back for this step
        h.err = 0;
        h.bad_dof = INT64_MAX;
        CK(cudaMemcpy(c->sc, &h, sizeof(h), cudaMemcpyHostToDevice));
        c->mlp.step_counter = counter0 + (int)ok_steps + 1;
        c->mlp.judge_this_step = false;
        if (int r2 = launch_step(c, end_time, false)) return r2;
        if (int r2 = sync_and_check(c)) return r2;
        done += ok_steps + 1;
    }
    return 0;
}

}  // namespace

extern "C" {

int plens_gpu_advance(plens_ctx* c, int64_t n_steps, double end_time)
{
    if (c && c->learned) {
        if (!c->dv.U || n_steps < 0) return PLENS_GPU_E_INVALID;
        if (!c->mlp.weights_set) return fail(c, PLENS_GPU_E_INVALID, "learned sensor: weights not set");
        return advance_learned(c, n_steps, end_time, nullptr);
    }
    if (int r = plens_gpu_advance_async(c, n_steps, end_time)) return r;
    return sync_and_check(c);
}

namespace {

// the copy streams, events and device buffers of plens_gpu_advance_states, once per context
int sequence_setup(plens_ctx* c)
{
    if (c->seq_in_buf) return 0;
    CK(cudaStreamCreateWithFlags(&c->seq_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->seq_out, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&c->seq_in_ready, &c->seq_in_free, &c->seq_out_ready, &c->seq_out_free})
        CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    double *a = nullptr, *b = nullptr;
    if (int r = dalloc(c, &a, 5 * c->nd)) return r;
    if (int r = dalloc(c, &b, 5 * c->nd)) return r;
    c->seq_in_buf = a;
    c->seq_out_buf = b;
    return 0;
}

// room for `count` member outcomes
int sequence_status(plens_ctx* c, int64_t count)
{
    if (count <= c->seq_status_cap) return 0;
    if (c->seq_status_host) cudaFreeHost(c->seq_status_host);
    c->seq_status_host = nullptr;
    c->seq_status_cap = 0;
    CK(cudaHostAlloc(reinterpret_cast<void**>(&c->seq_status_host), sizeof(MemberStatus) * count, cudaHostAllocMapped));
    CK(cudaHostGetDevicePointer(reinterpret_cast<void**>(&c->seq_status_dev), c->seq_status_host, 0));
    c->seq_status_cap = count;
    return 0;
}

// one member of a sequence: its state (staged in seq_in_buf) made current at time t0, its steps,
// its state copied to seq_out_buf and from there to the host on seq_out; the next member's copy
// into seq_in_buf is issued as soon as this member's state has left that buffer. Without the
// learned sensor nothing here waits for the GPU: the member's outcome goes to the mapped status
// array and the host goes on to enqueue the next member. The learned sensor's positivity
// fallback redoes a failed step from the host, so its members run one after the other.
int sequence_member(plens_ctx* c, int64_t j, int64_t count, const double* const* U_in, double* const* U_out,
                    double t0, int64_t n_steps, double end_time)
{
    const size_t bytes = sizeof(double) * 5 * c->nd;
    const unsigned grid = (unsigned)std::min<int64_t>((5 * c->nd + 255) / 256, 152 * 16);
    CK(cudaStreamWaitEvent(c->stream, c->seq_in_ready, 0));
    k_state_in<<<grid, 256, 0, c->stream>>>(c->dv, c->seq_in_buf);  // U and the FP32 image
    k_set_clock<<<1, 1, 0, c->stream>>>(c->dv, t0, 0);
    c->launches += 2;
    if (int r = check_launch(c, "state in")) return r;
    CK(cudaEventRecord(c->seq_in_free, c->stream));
    if (j + 1 < count) {
        CK(cudaStreamWaitEvent(c->seq_in, c->seq_in_free, 0));
        CK(cudaMemcpyAsync(c->seq_in_buf, U_in[j + 1], bytes, cudaMemcpyHostToDevice, c->seq_in));
        CK(cudaEventRecord(c->seq_in_ready, c->seq_in));
    }
    if (c->learned) {
        Scalars s0{};
        s0.time = t0;
        s0.n_steps = 0;
        if (int r = advance_learned(c, n_steps, end_time, &s0)) return r;
        const Scalars& h = *c->sc_host;  // synchronised: the mirror holds this member's clock
        c->seq_status_host[j] = MemberStatus{h.time, h.n_steps, h.bad_dof, 0, 0};
    } else {
        if (int r = plens_gpu_advance_async(c, n_steps, end_time)) return r;
        k_member_status<<<1, 1, 0, c->stream>>>(c->dv, c->seq_status_dev + j);
        c->launches += 1;
        if (int r = check_launch(c, "member status")) return r;
    }
    // the previous member's copy out must have left seq_out_buf
    CK(cudaStreamWaitEvent(c->stream, c->seq_out_free, 0));
    CK(cudaMemcpyAsync(c->seq_out_buf, c->dv.U, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaEventRecord(c->seq_out_ready, c->stream));
    CK(cudaStreamWaitEvent(c->seq_out, c->seq_out_ready, 0));
    CK(cudaMemcpyAsync(U_out[j], c->seq_out_buf, bytes, cudaMemcpyDeviceToHost, c->seq_out));
    CK(cudaEventRecord(c->seq_out_free, c->seq_out));
    return 0;
}

}  // namespace

int plens_gpu_advance_states(plens_ctx* c, int64_t count, const double* const* U_in, double* const* U_out,
                             double t0, int64_t n_steps, double end_time, double* t_out)
{
    if (!c || !c->dv.U) return PLENS_GPU_E_INVALID;
    if (count < 0 || n_steps < 0) return fail(c, PLENS_GPU_E_INVALID, "advance_states: negative count or step number");
    if (count == 0) return 0;
    if (!U_in || !U_out) return fail(c, PLENS_GPU_E_INVALID, "advance_states: null state array");
    for (int64_t j = 0; j < count; ++j)
        if (!U_in[j] || !U_out[j])
            return fail(c, PLENS_GPU_E_INVALID, "advance_states: null state buffer of member " + std::to_string(j));
    if (c->learned && !c->mlp.weights_set) return fail(c, PLENS_GPU_E_INVALID, "learned sensor: weights not set");
    if (int r = sequence_setup(c)) return r;
    if (int r = sequence_status(c, count)) return r;
    int r = 0;
    {
        const cudaError_t e = cudaMemcpyAsync(c->seq_in_buf, U_in[0], sizeof(double) * 5 * c->nd,
                                              cudaMemcpyHostToDevice, c->seq_in);
        r = (e == cudaSuccess) ? 0 : cuda_fail(c, e, "advance_states: copy in");
        if (!r) {
            const cudaError_t e2 = cudaEventRecord(c->seq_in_ready, c->seq_in);
            if (e2 != cudaSuccess) r = cuda_fail(c, e2, "advance_states: event");
        }
    }
    int64_t j = 0;
    for (; j < count && !r; ++j) r = sequence_member(c, j, count, U_in, U_out, t0, n_steps, end_time);
    // no copy into or out of the caller's buffers outlives the call
    const cudaError_t es = cudaStreamSynchronize(c->stream);
    const cudaError_t ei = cudaStreamSynchronize(c->seq_in);
    const cudaError_t eo = cudaStreamSynchronize(c->seq_out);
    if (r) {
        c->err = "advance_states: member " + std::to_string(j - 1) + ": " + c->err;
        return r;
    }
    if (es != cudaSuccess) return cuda_fail(c, es, "advance_states: steps");
    if (ei != cudaSuccess) return cuda_fail(c, ei, "advance_states: copy in");
    if (eo != cudaSuccess) return cuda_fail(c, eo, "advance_states: copy out");
    for (int64_t k = 0; k < count; ++k) {
        const MemberStatus m = c->seq_status_host[k];
        if (m.err == PLENS_GPU_E_POSITIVITY) {
            c->bad_dof_host = m.bad_dof;
            return fail(c, PLENS_GPU_E_POSITIVITY, "advance_states: member " + std::to_string(k) +
                                                       ": Positivity assertion failed at dof " + std::to_string(m.bad_dof));
        }
        if (m.err) return fail(c, m.err, "advance_states: member " + std::to_string(k) + ": device error " + std::to_string(m.err));
    }
    if (t_out)
        for (int64_t k = 0; k < count; ++k) t_out[k] = c->seq_status_host[k].time;
    return 0;
}

int plens_gpu_error_norms(plens_ctx* c, double* ss_error, double* conv_error)
{
    if (!c) return PLENS_GPU_E_INVALID;
    if ((ss_error && !c->prm.calc_ss_error) || (conv_error && !c->prm.calc_conv_error))
        return fail(c, PLENS_GPU_E_INVALID, "error norm not requested at setup");
    if (!ss_error && !conv_error) return 0;
    cudaStream_t st = c->stream;
    // the time step of the current state: write() runs at stage 1 after calc_time_step
    k_step_begin<<<1, 1, 0, st>>>(c->dv, 1e300);
    c->launches += 1;
    if (int r = launch_time_step(c)) return r;
    const int expr = c->prm.calc_conv_error ? c->prm.expr_conv_exact : -1;
    const unsigned threads = (unsigned)(((c->P * c->P * c->P) + 31) / 32 * 32);
    switch (c->P) {
    case 2: k_cell_errors<2><<<(unsigned)c->nc, threads, 0, st>>>(c->dv, c->gi, c->rhoE_old, c->q_wJ, c->q_xyz, expr, c->err_cell); break;
    case 3: k_cell_errors<3><<<(unsigned)c->nc, threads, 0, st>>>(c->dv, c->gi, c->rhoE_old, c->q_wJ, c->q_xyz, expr, c->err_cell); break;
    case 4: k_cell_errors<4><<<(unsigned)c->nc, threads, 0, st>>>(c->dv, c->gi, c->rhoE_old, c->q_wJ, c->q_xyz, expr, c->err_cell); break;
    case 5: k_cell_errors<5><<<(unsigned)c->nc, threads, 0, st>>>(c->dv, c->gi, c->rhoE_old, c->q_wJ, c->q_xyz, expr, c->err_cell); break;
    default: k_cell_errors<6><<<(unsigned)c->nc, threads, 0, st>>>(c->dv, c->gi, c->rhoE_old, c->q_wJ, c->q_xyz, expr, c->err_cell); break;
    }
    k_sum_errors<<<1, 1024, 0, st>>>(c->err_cell, c->nc, c->err_sum);
    c->launches += 2;
    if (int r = check_launch(c, "error norm kernels")) return r;
    double h[3];
    CK(cudaMemcpyAsync(h, c->err_sum, sizeof(h), cudaMemcpyDeviceToHost, st));
    if (int r = sync_and_check(c)) return r;
    if (ss_error) *ss_error = std::sqrt(h[1]) / std::sqrt(h[0]);
    if (conv_error) *conv_error = std::sqrt(h[2]);
    return 0;
}

int plens_gpu_get_cell_scalars(plens_ctx* c, double* alpha, double* alpha_d, double* dt_cell)
{
    if (!c) return PLENS_GPU_E_INVALID;
    CK(cudaStreamSynchronize(c->stream));
    if (alpha) CK(cudaMemcpy(alpha, c->dv.alpha, sizeof(double) * c->nc, cudaMemcpyDeviceToHost));
    if (alpha_d) CK(cudaMemcpy(alpha_d, c->dv.alpha_d, sizeof(double) * c->nc, cudaMemcpyDeviceToHost));
    if (dt_cell && c->dv.dt_loc) {
        CK(cudaMemcpy(dt_cell, c->dv.dt_loc, sizeof(double) * c->nc, cudaMemcpyDeviceToHost));
    } else if (dt_cell) {
        Scalars h;
        if (int r = read_scalars(c, &h)) return r;
        for (int64_t i = 0; i < c->nc; ++i) dt_cell[i] = h.dt_update;
    }
    return 0;
}

int plens_gpu_troubled_cells(plens_ctx* c, int32_t* cells, int64_t* count)
{
    if (!c || !count) return PLENS_GPU_E_INVALID;
    if (!c->dv.lo_list) return fail(c, PLENS_GPU_E_INVALID, "this context has no compacted troubled-cell list");
    CK(cudaStreamSynchronize(c->stream));
    int32_t n = 0;
    CK(cudaMemcpy(&n, c->dv.lo_count, sizeof(n), cudaMemcpyDeviceToHost));
    *count = n;
    if (cells && n > 0) CK(cudaMemcpy(cells, c->dv.lo_list, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    return 0;
}

int plens_gpu_get_avars(plens_ctx* c, double* avars)
{
    if (!c || !avars) return PLENS_GPU_E_INVALID;
    if (!c->viscous) return fail(c, PLENS_GPU_E_INVALID, "inviscid run has no auxiliary variables");
    CK(cudaStreamSynchronize(c->stream));
    if (c->mixed) {  // the mixed form keeps them in FP32
        std::vector<float> f((size_t)(9 * c->nd));
        CK(cudaMemcpy(f.data(), c->dv.avars, sizeof(float) * 9 * c->nd, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < f.size(); ++i) avars[i] = f[i];
        return 0;
    }
    CK(cudaMemcpy(avars, c->dv.avars, sizeof(double) * 9 * c->nd, cudaMemcpyDeviceToHost));
    return 0;
}

namespace {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

__global__ void k_selftest_conversions(int64_t n, unsigned long long seed, unsigned long long* bad)
{
    unsigned long long nbad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long h = splitmix64(seed + (unsigned long long)i);
        unsigned long long b = h;
        const int mode = (int)(i & 3);
        if (mode) {  // exponent in [860, 1160): around and inside the normal float range
            const unsigned long long e = 860 + (h >> 52) % 300;
            b = (h & 0x800fffffffffffffULL) | (e << 52);
            if (mode == 2) b = (b & ~0x1fffffffULL) | 0x10000000ULL;                       // exact tie
            if (mode == 3) b = (b & ~0x1fffffffULL) | ((h & 1) ? 0x0fffffffULL : 0x10000001ULL);  // near tie
        }
        const double x = __longlong_as_double((long long)b);
        const float a = f64_to_f32(x), r = __double2float_rn(x);
        const bool ok1 = (a != a) ? (r != r) : (__float_as_uint(a) == __float_as_uint(r));
        const float xf = __uint_as_float((unsigned int)(h >> 32));
        const double c = f32_to_f64(xf), d = (double)xf;
        const bool ok2 = (c != c) ? (d != d) : (__double_as_longlong(c) == __double_as_longlong(d));
        nbad += (ok1 ? 0 : 1) + (ok2 ? 0 : 1);
    }
    if (nbad) atomicAdd(bad, nbad);
}

}  // namespace

int plens_gpu_selftest_conversions(int64_t n, uint64_t seed, int64_t* mismatches)
{
    if (n < 0 || !mismatches) return PLENS_GPU_E_INVALID;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return PLENS_GPU_E_CUDA;
    unsigned long long h = 0;
    cudaMemset(d, 0, sizeof(*d));
    k_selftest_conversions<<<152 * 4, 256>>>(n, seed, d);
    const cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return PLENS_GPU_E_CUDA;
    *mismatches = (int64_t)h;
    return 0;
}

namespace {
// snapshot layout: U [5][nd] f64 | alpha [nc] f64 | alpha_d [nc] f64 | avars (viscous: [9][nd] in
// the form's storage type) | Scalars
size_t snap_off_avars(const plens_ctx* c) { return sizeof(double) * (5 * c->nd + 2 * c->nc); }
size_t snap_avars_bytes(const plens_ctx* c)
{
    return c->viscous ? (c->mixed ? sizeof(float) : sizeof(double)) * 9 * c->nd : 0;
}
size_t snap_off_scalars(const plens_ctx* c) { return (snap_off_avars(c) + snap_avars_bytes(c) + 15) / 16 * 16; }
}  // namespace

int plens_gpu_set_sensor_tensor_cores(plens_ctx* c, int enable)
{
    if (!c) return PLENS_GPU_E_INVALID;
    if (!c->learned) return fail(c, PLENS_GPU_E_INVALID, "context was created without the learned sensor");
    if (int r = sync_and_check(c)) return r;
    c->mlp.use_tc = enable != 0;
    for (auto& gx : c->step_graph)  // the step's launch sequence changed
        if (gx) {
            cudaGraphExecDestroy(gx);
            gx = nullptr;
        }
    return 0;
}

int plens_gpu_set_indicator_tensor_cores(plens_ctx* c, int enable)
{
    if (!c) return PLENS_GPU_E_INVALID;
    if (!c->cbm_tc) return fail(c, PLENS_GPU_E_INVALID, "the tensor-core modal indicator needs a mixed-precision context of degree 3");
    if (c->learned) return fail(c, PLENS_GPU_E_INVALID, "context uses the learned sensor, not the modal indicator");
    if (int r = sync_and_check(c)) return r;
    c->indicator_tc = enable != 0;
    for (auto& gx : c->step_graph)  // the step's launch sequence changed
        if (gx) {
            cudaGraphExecDestroy(gx);
            gx = nullptr;
        }
    return 0;
}

int plens_gpu_set_list_decoding(plens_ctx* c, int enable)
{
    if (!c) return PLENS_GPU_E_INVALID;
    if (!c->dv.lo_blk) return fail(c, PLENS_GPU_E_INVALID, "this context has no compacted troubled-cell list");
    if (enable && (c->nc + kSmoothThreads - 1) / kSmoothThreads + 1 > kLoDecodeMaxBlocks)
        return fail(c, PLENS_GPU_E_INVALID, "the mesh's block counts do not fit the subcell kernel's shared memory");
    if (int r = sync_and_check(c)) return r;
    c->dv.lo_decode = enable ? 1 : 0;
    for (auto& gx : c->step_graph)  // the step's launch sequence and kernel arguments changed
        if (gx) {
            cudaGraphExecDestroy(gx);
            gx = nullptr;
        }
    return 0;
}

int plens_gpu_snapshot_begin(plens_ctx* c)
{
    if (!c || !c->dv.U) return PLENS_GPU_E_INVALID;
    if (c->snap_pending) return fail(c, PLENS_GPU_E_INVALID, "a snapshot is already pending");
    if (!c->snap_dev) {
        c->snap_bytes = snap_off_scalars(c) + sizeof(Scalars);
        CK(cudaMalloc(&c->snap_dev, c->snap_bytes));
        CK(cudaMallocHost(&c->snap_host, c->snap_bytes));
        CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->snap_ready, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->snap_done, cudaEventDisableTiming));
    }
    cudaStream_t st = c->stream;
    unsigned char* d = c->snap_dev;
    CK(cudaMemcpyAsync(d, c->dv.U, sizeof(double) * 5 * c->nd, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(d + sizeof(double) * 5 * c->nd, c->dv.alpha, sizeof(double) * c->nc, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(d + sizeof(double) * (5 * c->nd + c->nc), c->dv.alpha_d, sizeof(double) * c->nc,
                       cudaMemcpyDeviceToDevice, st));
    if (c->viscous)
        CK(cudaMemcpyAsync(d + snap_off_avars(c), c->dv.avars, snap_avars_bytes(c), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(d + snap_off_scalars(c), c->sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, st));
    CK(cudaEventRecord(c->snap_ready, st));
    CK(cudaStreamWaitEvent(c->copy_stream, c->snap_ready, 0));
    CK(cudaMemcpyAsync(c->snap_host, c->snap_dev, c->snap_bytes, cudaMemcpyDeviceToHost, c->copy_stream));
    CK(cudaEventRecord(c->snap_done, c->copy_stream));
    c->snap_pending = true;
    return 0;
}

int plens_gpu_snapshot_end(plens_ctx* c, double* U, double* alpha, double* alpha_d, double* avars, double* time,
                           int64_t* n_steps, double* dt)
{
    if (!c) return PLENS_GPU_E_INVALID;
    if (!c->snap_pending) return fail(c, PLENS_GPU_E_INVALID, "no snapshot pending");
    c->snap_pending = false;
    CK(cudaEventSynchronize(c->snap_done));
    const unsigned char* h = c->snap_host;
    if (U) std::memcpy(U, h, sizeof(double) * 5 * c->nd);
    if (alpha) std::memcpy(alpha, h + sizeof(double) * 5 * c->nd, sizeof(double) * c->nc);
    if (alpha_d) std::memcpy(alpha_d, h + sizeof(double) * (5 * c->nd + c->nc), sizeof(double) * c->nc);
    if (avars && c->viscous) {
        if (c->mixed) {
            const float* f = reinterpret_cast<const float*>(h + snap_off_avars(c));
            for (int64_t i = 0; i < 9 * c->nd; ++i) avars[i] = f[i];
        } else {
            std::memcpy(avars, h + snap_off_avars(c), sizeof(double) * 9 * c->nd);
        }
    }
    Scalars sc;
    std::memcpy(&sc, h + snap_off_scalars(c), sizeof(sc));
    if (time) *time = sc.time;
    if (n_steps) *n_steps = sc.n_steps;
    if (dt) *dt = sc.dt;
    return 0;
}

int plens_gpu_first_bad_dof(const plens_ctx* c, int64_t* dof)
{
    if (!c || !dof) return PLENS_GPU_E_INVALID;
    *dof = c->bad_dof_host;
    return 0;
}

int plens_gpu_set_sensor_weights(plens_ctx* c, const float* params)
{
    if (!c || !params) return PLENS_GPU_E_INVALID;
    if (!c->learned) return fail(c, PLENS_GPU_E_INVALID, "context was created without the learned sensor");
    if (mlp_set_weights(c->mlp, params, c->stream)) return fail(c, PLENS_GPU_E_CUDA, "weight upload");
    return 0;
}

int plens_gpu_sensor_stats(plens_ctx* c, int64_t* judged, int64_t* fallbacks, double* max_alpha_err, int64_t* lo_cells)
{
    if (!c) return PLENS_GPU_E_INVALID;
    Scalars h;
    if (int r = read_scalars(c, &h)) return r;
    if (judged) *judged = h.judged;
    if (fallbacks) *fallbacks = h.fallbacks;
    if (max_alpha_err) *max_alpha_err = h.max_alpha_err;
    if (lo_cells) {
        int32_t n = 0;
        if (c->dv.lo_count) CK(cudaMemcpy(&n, c->dv.lo_count, sizeof(n), cudaMemcpyDeviceToHost));
        *lo_cells = n;
    }
    return 0;
}

int plens_gpu_sensor_pairs(plens_ctx* c, float* x, float* y)
{
    if (!c || !x || !y) return PLENS_GPU_E_INVALID;
    if (int r = mlp_pairs(c->dv, c->ops, c->gas, c->bp, c->P, x, y, c->stream, c->launches)) return fail(c, r, "sensor pairs");
    return 0;
}

}  // extern "C"
