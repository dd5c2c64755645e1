// noalloc.cu -- stable time step of a caller-owned state without any device allocation.
//
// Who needs this: callers that are not allowed to allocate device memory -- for example a host
// framework that owns all GPU memory through its own pool and forbids libraries from calling
// cudaMalloc, or code that must not allocate between two points of a run (allocation can
// synchronise the device and perturb a measured or real-time loop). The context entry points
// (plens_gpu_create / plens_gpu_time_step) allocate their buffers; this one does not.
//
// The per-cell stable steps (the reference's loc_time_steps) live in a file-scope __device__
// array of PLENS_GPU_NOALLOC_MAX_CELLS doubles (2 MiB), which every GPU that loads the library
// holds until the process exits. All calls share that array and it keeps the last call's
// contents; every call writes each cell it reads before reading it, so nothing needs clearing,
// but calls that overlap on the GPU (on different streams, or from several threads) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "device.cuh"
#include "flux.cuh"
#include "plens_gpu.h"

namespace {

using namespace plens_gpu;

static __device__ __align__(256) double g_noalloc_cell_dt[PLENS_GPU_NOALLOC_MAX_CELLS];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch[kMaxDevices] = {};

// Message of the last failed call on this thread, read through plens_gpu_last_error(NULL).
thread_local std::string g_noalloc_err = "no error";

int noalloc_fail(int code, const std::string& msg)
{
    g_noalloc_err = "plens_gpu_time_step_noalloc: " + msg;
    return code;
}

// Device address of the scratch array on the current device. Host code must not pass
// g_noalloc_cell_dt itself to a kernel: on the host that name is only a stand-in.
int scratch_on_current_device(double** out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PLENS_GPU_E_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch[dev]) {
        double* p = nullptr;
        if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_cell_dt) != cudaSuccess || !p)
            return PLENS_GPU_E_CUDA;
        g_scratch[dev] = p;
    }
    *out = g_scratch[dev];
    return PLENS_GPU_OK;
}

struct NoallocGas {
    double gamma, R, mu0, T0, S, N15;
    int const_visc, inviscid, N, P3;
};

// Pass 1: one thread per dof, the per-cell minimum of the stable step (the per-dof formula of
// PLENS::calc_time_step, dgsem/plens.cc:3839-3864) into the scratch array.
__global__ void __launch_bounds__(256) k_cell_dt_noalloc(const double* __restrict__ U, const double* __restrict__ Jinv,
                                                         const double* __restrict__ h_min, int64_t nc, NoallocGas g,
                                                         double courant, double* __restrict__ cell_dt)
{
    __shared__ double s_dt[256];
    const int P3 = g.P3;
    const int cells_per_block = 256 / P3;
    const int cl = threadIdx.x / P3, node = threadIdx.x - cl * P3;
    const int64_t cell = (int64_t)blockIdx.x * cells_per_block + cl;
    const bool valid = cl < cells_per_block && cell < nc;
    const int64_t nd = nc * P3;
    double cur = 1e6;
    if (valid) {
        const int64_t dof = cell * P3 + node;
        double cs[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) cs[v] = U[v * nd + dof];
        const double a = sqrt(g.gamma * get_p(cs, g.gamma) / cs[0]);
        const double vel[3] = {cs[1] / cs[0], cs[2] / cs[0], cs[3] / cs[0]};
        double madv = 0;
#pragma unroll
        for (int row = 0; row < 3; ++row) {
            double acc = 0.0;
#pragma unroll
            for (int col = 0; col < 3; ++col) acc += Jinv[(col * 3 + row) * nd + dof] * vel[col];
            madv = (row == 0 || acc > madv) ? acc : madv;
        }
        double mu = 0.0;
        if (!g.inviscid) {
            const double T = get_e(cs) / (g.R / (g.gamma - 1));
            mu = g.const_visc ? g.mu0 : g.mu0 * pow(T / g.T0, 1.5) * (g.T0 + g.S) / (T + g.S);
        }
        const double h = h_min[cell];
        const double step = courant / (g.N15 * (madv + a / h + (double)(g.N * g.N) * mu / (h * h * cs[0])));
        if (step < cur) cur = step;
    }
    s_dt[threadIdx.x] = cur;
    __syncthreads();
    if (valid && node == 0) {
        double m = 1e6;
        for (int k = 0; k < P3; ++k) {
            const double v = s_dt[cl * P3 + k];
            if (v < m) m = v;
        }
        cell_dt[cell] = m;
    }
}

// Pass 2: one block, min over the cells (warp shuffles, then across warps).
__global__ void __launch_bounds__(1024) k_global_dt_noalloc(const double* __restrict__ cell_dt, int64_t nc, double* __restrict__ dt_out)
{
    __shared__ double s_w[32];
    double m = 1e6;
    for (int64_t c = threadIdx.x; c < nc; c += blockDim.x) {
        const double v = cell_dt[c];
        if (v < m) m = v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, m, off);
        if (o < m) m = o;
    }
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = s_w[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (s_w[w] < r) r = s_w[w];
        *dt_out = r;
    }
}

}  // namespace

extern "C" int plens_gpu_time_step_noalloc(const double* U, const double* Jinv, const double* h_min, int64_t n_cells,
                                           int32_t degree, const plens_params* params, double courant, double* dt_out,
                                           void* stream)
{
    if (!U || !Jinv || !h_min || !params || !dt_out) return noalloc_fail(PLENS_GPU_E_INVALID, "null pointer argument");
    if (degree < 1 || degree > 5) return noalloc_fail(PLENS_GPU_E_INVALID, "degree must lie in [1,5]");
    if (n_cells <= 0) return noalloc_fail(PLENS_GPU_E_INVALID, "n_cells must be positive");
    if (n_cells > PLENS_GPU_NOALLOC_MAX_CELLS)
        return noalloc_fail(PLENS_GPU_E_INVALID, "n_cells = " + std::to_string(n_cells) + " exceeds the scratch array (" +
                                                     std::to_string(PLENS_GPU_NOALLOC_MAX_CELLS) + " cells)");
    // an error left by earlier work is reported as it is (not cleared), so that the launch check
    // below sees only this call's launches
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
        return noalloc_fail(PLENS_GPU_E_CUDA, std::string("a CUDA error is pending from earlier work: ") + cudaGetErrorString(pending));
    double* scratch = nullptr;
    if (scratch_on_current_device(&scratch)) return noalloc_fail(PLENS_GPU_E_CUDA, "scratch array address lookup failed");
    NoallocGas g;
    g.gamma = params->gamma;
    g.R = params->R;
    g.mu0 = params->mu0;
    g.T0 = params->T0;
    g.S = params->S;
    g.N = degree;
    g.P3 = (degree + 1) * (degree + 1) * (degree + 1);
    g.N15 = std::pow(degree, 1.5);
    g.const_visc = params->const_viscosity;
    g.inviscid = params->mu0 < 1e-16 ? 1 : 0;
    const double co = (courant >= 1) ? 0.9 : courant;  // calc_time_step caps Co >= 1 to 0.9
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int cpb = 256 / g.P3;
    const int64_t blocks = (n_cells + cpb - 1) / cpb;
    k_cell_dt_noalloc<<<(unsigned)blocks, 256, 0, st>>>(U, Jinv, h_min, n_cells, g, co, scratch);
    k_global_dt_noalloc<<<1, 1024, 0, st>>>(scratch, n_cells, dt_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(PLENS_GPU_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return PLENS_GPU_OK;
}

// plens_gpu_last_error(NULL): the message of the last failed context-free call on this thread
extern "C" __attribute__((visibility("hidden"))) const char* plens_gpu_noalloc_last_error_message()
{
    return g_noalloc_err.c_str();
}
