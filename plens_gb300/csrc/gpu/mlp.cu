// mlp.cu -- learned troubled-cell sensor: fused inference + troubled-cell compaction inside the
// RHS, the judge/fallback logic, training-pair extraction, and the training kernels (forward,
// backward, Adam) behind plens_gpu_mlp_train / _loss_grad / _infer. FP32 throughout.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "blender_tc.cuh"
#include "kernels.cuh"
#include "mlp.cuh"
#include "mlp_tc.cuh"

namespace plens_gpu {

namespace {

// 1D Lagrange interpolation from the P GLL nodes to the 4 GLL nodes of [0,1] (exact for
// polynomials of degree <= 3, so N = 2 data is represented without loss).
struct Interp {
    float I[4 * kMaxP];
    int P;
};

void host_gll(int n, std::vector<double>& x)
{
    const int N = n - 1;
    std::vector<long double> t(n);
    for (int i = 0; i < n; ++i) t[i] = std::cos(M_PI * (long double)i / N);
    for (int it = 0; it < 200; ++it) {
        for (int i = 0; i < n; ++i) {
            long double a = 1, b = t[i];
            for (int k = 2; k <= N; ++k) { const long double c = ((2 * k - 1) * t[i] * b - (k - 1) * a) / k; a = b; b = c; }
            if (N == 1) a = 1;
            t[i] = t[i] - (t[i] * b - a) / (n * b);
        }
    }
    x.assign(n, 0);
    for (int i = 0; i < n; ++i) x[n - 1 - i] = (double)((t[i] + 1) / 2);
    x[0] = 0;
    x[n - 1] = 1;
}

Interp make_interp(int P)
{
    Interp r;
    std::memset(&r, 0, sizeof(r));
    r.P = P;
    std::vector<double> xs, x4;
    host_gll(P, xs);
    host_gll(4, x4);
    for (int a = 0; a < 4; ++a)
        for (int i = 0; i < P; ++i) {
            double l = 1;
            for (int m = 0; m < P; ++m)
                if (m != i) l *= (x4[a] - xs[m]) / (xs[i] - xs[m]);
            r.I[a * kMaxP + i] = (float)l;
        }
    return r;
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x)
{
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// rho*p at the P^3 nodes (vs) -> interpolated to the 4^3 GLL nodes, divided by its mean, minus 1
// (xs); one warp.
template <int P, int XS = 1>
__device__ void interp_normalise(const Interp& ip, float* vs, float* ts, float* xs)
{
    constexpr int P2 = P * P;
    const int lane = threadIdx.x & 31;
    if (P == 4) {
        for (int n = lane; n < 64; n += 32) xs[n * XS] = vs[n];
    } else {
        // x: [a][j][k] (a < 4), then y, then z
        for (int n = lane; n < 4 * P2; n += 32) {
            const int a = n % 4, j = (n / 4) % P, k = n / (4 * P);
            float s = 0;
            for (int i = 0; i < P; ++i) s += ip.I[a * kMaxP + i] * vs[i + P * j + P2 * k];
            ts[n] = s;  // layout a + 4 j + 4P k
        }
        __syncwarp();
        for (int n = lane; n < 16 * P; n += 32) {
            const int a = n % 4, b = (n / 4) % 4, k = n / 16;
            float s = 0;
            for (int j = 0; j < P; ++j) s += ip.I[b * kMaxP + j] * ts[a + 4 * j + 4 * P * k];
            vs[n] = s;  // layout a + 4 b + 16 k
        }
        __syncwarp();
        for (int n = lane; n < 64; n += 32) {
            const int a = n % 4, b = (n / 4) % 4, cc = n / 16;
            float s = 0;
            for (int k = 0; k < P; ++k) s += ip.I[cc * kMaxP + k] * vs[a + 4 * b + 16 * k];
            xs[n * XS] = s;
        }
    }
    __syncwarp();
    float m = xs[lane * XS] + xs[(lane + 32) * XS];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m += __shfl_xor_sync(0xffffffffu, m, off);
    m *= (1.0f / 64.0f);
    const float inv = 1.0f / m;
    xs[lane * XS] = xs[lane * XS] * inv - 1.0f;
    xs[(lane + 32) * XS] = xs[(lane + 32) * XS] * inv - 1.0f;
    __syncwarp();
}


// Features of one cell into xs[64] (shared): rho*p at the nodes, interpolated to 4^3 GLL nodes,
// normalised by its mean. Executed by one warp. The state is read once here, so the positivity
// assertion of the RHS (dgsem/plens.cc:2531-2546) is made here too, with the FP64 decision of the
// mixed form.
template <int P>
__device__ void cell_features(const Dev& dv, double gamma, const Interp& ip, int64_t cell, float* vs, float* ts, float* xs)
{
    constexpr int P2 = P * P, P3 = P2 * P;
    const int lane = threadIdx.x & 31;
    const float gm = f64_to_f32(gamma);
    for (int n = lane; n < P3; n += 32) {
        const int64_t dof = cell * P3 + n;
        float cf[5];
        bool ok;
        if (dv.Uf) {  // mixed form: the FP32 image of the state
            load_state<float>(dv, dof, cf);
            ok = positive_dof_screened(dv, dof, cf);
        } else {
            double c[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                c[v] = dv.U[v * dv.nd + dof];
                cf[v] = f64_to_f32(c[v]);
            }
            ok = positive_state_screened(c, cf);
        }
        if (!ok) {
            atomicMin(&dv.sc->bad_dof, (long long)dof);
            dv.sc->err = PLENS_GPU_E_POSITIVITY;
        }
        vs[n] = get_p(cf, gm) * cf[0];
    }
    __syncwarp();
    interp_normalise<P>(ip, vs, ts, xs);
}

// MLP forward (W1 and W2 stored transposed, [in][out], so the 32 lanes -- each computing two
// outputs -- read consecutive shared-memory words) for G cells at once by one warp: the inputs are stored [k][g] so one
// 16-byte broadcast load feeds the G cells, and each weight read from shared memory serves G
// multiply-adds (the per-cell form reads one weight per multiply-add).
template <int G>
__device__ void mlp_forward_group(const float* W, const float* xs, float* hs, float amax, float out[G])
{
    static_assert(G == 4, "inputs are read as float4");
    const int lane = threadIdx.x & 31;
    const float* W1t = W;
    const float* b1 = W1t + kMlpHid * kMlpIn;
    const float* W2t = b1 + kMlpHid;
    const float* b2 = W2t + kMlpHid * kMlpHid;
    const float* w3 = b2 + kMlpHid;
    const float b3 = w3[kMlpHid];
    float h0[G], h1[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
        h0[g] = b1[lane];
        h1[g] = b1[lane + 32];
    }
#pragma unroll 8
    for (int k = 0; k < kMlpIn; ++k) {
        const float4 x = *reinterpret_cast<const float4*>(xs + k * G);
        const float w0 = W1t[k * kMlpHid + lane], w1 = W1t[k * kMlpHid + lane + 32];
        h0[0] += w0 * x.x; h0[1] += w0 * x.y; h0[2] += w0 * x.z; h0[3] += w0 * x.w;
        h1[0] += w1 * x.x; h1[1] += w1 * x.y; h1[2] += w1 * x.z; h1[3] += w1 * x.w;
    }
    __syncwarp();
#pragma unroll
    for (int g = 0; g < G; ++g) {
        hs[lane * G + g] = gelu(h0[g]);
        hs[(lane + 32) * G + g] = gelu(h1[g]);
    }
    __syncwarp();
#pragma unroll
    for (int g = 0; g < G; ++g) {
        h0[g] = b2[lane];
        h1[g] = b2[lane + 32];
    }
#pragma unroll 8
    for (int k = 0; k < kMlpHid; ++k) {
        const float4 x = *reinterpret_cast<const float4*>(hs + k * G);
        const float w0 = W2t[k * kMlpHid + lane], w1 = W2t[k * kMlpHid + lane + 32];
        h0[0] += w0 * x.x; h0[1] += w0 * x.y; h0[2] += w0 * x.z; h0[3] += w0 * x.w;
        h1[0] += w1 * x.x; h1[1] += w1 * x.y; h1[2] += w1 * x.z; h1[3] += w1 * x.w;
    }
#pragma unroll
    for (int g = 0; g < G; ++g) {
        float z = w3[lane] * gelu(h0[g]) + w3[lane + 32] * gelu(h1[g]);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) z += __shfl_xor_sync(0xffffffffu, z, off);
        out[g] = amax / (1.0f + expf(-(z + b3)));
    }
    __syncwarp();
}

constexpr int kWarpsPerBlock = 8;
constexpr int kGroup = 4;  // cells per warp in one network evaluation

// Learned values below this are set to 0 (the modal indicator's own cut is alpha_min = 1e-3): the
// network's sigmoid never returns exact zeros, and without a cut the subcell residual would run
// on every smooth cell. The judge bounds the error this introduces.
constexpr float kLearnedCut = 0.01f;

// Per-warp shared scratch of the inference kernel (floats): nodal values, interpolation / modal
// transform buffer, network input, hidden layer.
template <int P>
struct InferScratch {
    // nodal values / y-pass output / modal transform buffers, then the group's inputs and hidden layer
    static constexpr int V0 = P * P * P, V1 = 16 * P, V2 = 4 * P * P;
    static constexpr int V = ((V0 > V1 ? (V0 > V2 ? V0 : V2) : (V1 > V2 ? V1 : V2)) + 3) / 4 * 4;
    static constexpr int per_warp = 2 * V + 2 * 64 * kGroup;
};
constexpr int kParamsPad = (kMlpParams + 3) / 4 * 4;  // float4 copies

// This cell's FP32 state, the nodes lane, lane + 32, ... of the warp (NPL per lane).
template <int P, int NPL>
__device__ __forceinline__ void load_cell_f32(const Dev& dv, int64_t cell, int lane, float u[NPL][5])
{
    constexpr int P3 = P * P * P;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        const int n = lane + 32 * j;
        if (n < P3) {
            if (dv.Uf) {
                load_state<float>(dv, cell * P3 + n, u[j]);
            } else {  // FP64 form with the learned sensor: convert the state
#pragma unroll
                for (int v = 0; v < 5; ++v) u[j][v] = f64_to_f32(dv.U[v * dv.nd + cell * P3 + n]);
            }
        }
    }
}

// The plain modal indicator of one cell by one warp in FP32 (the mixed form's k_blender: variable,
// separable nodal -> modal transform, mode energies, Hennemann alpha), for the cells the judge
// handed back; returns alpha before the wall override.
template <int P, int NPL>
__device__ float modal_alpha_warp(const Ops& ops, const BlendP& bp, float gm, const float u[NPL][5], float* a, float* b)
{
    constexpr int P2 = P * P, P3 = P2 * P, N = P - 1;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        const int n = lane + 32 * j;
        if (n < P3) {
            const float p = get_p(u[j], gm);
            a[n] = (bp.var == 2) ? u[j][0] : (bp.var == 1) ? p : p * u[j][0];
        }
    }
    __syncwarp();
    for (int n = lane; n < P3; n += 32) {
        const int i = n % P, j = (n / P) % P, k = n / P2;
        float acc = 0;
        for (int m = 0; m < P; ++m) acc += ops.fC1[i * P + m] * a[m + P * j + P2 * k];
        b[n] = acc;
    }
    __syncwarp();
    for (int n = lane; n < P3; n += 32) {
        const int i = n % P, j = (n / P) % P, k = n / P2;
        float acc = 0;
        for (int m = 0; m < P; ++m) acc += ops.fC1[j * P + m] * b[i + P * m + P2 * k];
        a[n] = acc;
    }
    __syncwarp();
    float e0 = 0, e1 = 0, e2 = 0;
    for (int n = lane; n < P3; n += 32) {
        const int i = n % P, j = (n / P) % P, k = n / P2;
        float md = 0;
        for (int m = 0; m < P; ++m) md += ops.fC1[k * P + m] * a[i + P * j + P2 * m];
        const float e = md * md;
        e0 += e;
        if (i < N && j < N && k < N) e1 += e;
        if (i < N - 1 && j < N - 1 && k < N - 1) e2 += e;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        e0 += __shfl_xor_sync(0xffffffffu, e0, off);
        e1 += __shfl_xor_sync(0xffffffffu, e1, off);
        e2 += __shfl_xor_sync(0xffffffffu, e2, off);
    }
    __syncwarp();
    float trouble = 1.0f - __fdividef(e1, e0);
    if (N > 2) {
        const float t2 = 1.0f - __fdividef(e2, e1);
        if (t2 > trouble) trouble = t2;
    }
    const float thr = f64_to_f32(bp.thr), amin = f64_to_f32(bp.amin), amax = f64_to_f32(bp.amax);
    if (bp.func == 0) {
        const float at = __fdividef(1.0f, 1.0f + __expf(-f64_to_f32(bp.sharp) * (__fdividef(trouble, thr) - 1.0f)));
        return (at < amin) ? 0.0f : (at < amax ? at : amax);
    }
    const float at = __fdividef(trouble, thr);
    return (at > 1.0f) ? 1.0f : at;
}

// Network input of one cell from its FP32 state (rho*p at the nodes, interpolated to 4^3 GLL
// nodes, normalised by the mean), with the positivity assertion of the RHS.
template <int P, int NPL, int XS = 1>
__device__ void features_from_state(const Dev& dv, int64_t cell, float gm, const Interp& ip, const float u[NPL][5],
                                    float* vs, float* ts, float* xs)
{
    constexpr int P2 = P * P, P3 = P2 * P;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        const int n = lane + 32 * j;
        if (n < P3) {
            const int64_t dof = cell * P3 + n;
            if (!positive_dof_screened(dv, dof, u[j])) {
                atomicMin(&dv.sc->bad_dof, (long long)dof);
                dv.sc->err = PLENS_GPU_E_POSITIVITY;
            }
            vs[n] = get_p(u[j], gm) * u[j][0];
        }
    }
    __syncwarp();
    interp_normalise<P, XS>(ip, vs, ts, xs);
}

// Fused inference of the modal indicator's value (the blender before neighbour smoothing):
// features, MLP, cut, wall override; with `use_mask`, the cells the judge handed back get the
// plain indicator instead, computed by the same warp. Persistent grid: each warp walks cells
// with a stride and holds the next cell's state in registers while it evaluates the current one.
template <int P>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, (P <= 4 ? 3 : 1)) k_sensor_infer(Dev dv, const float* __restrict__ Wt, GasP g,
                                                                       BlendP bp, Ops ops, Interp ip, double* out,
                                                                       int gated, const uint8_t* mask)
{
    constexpr int P3 = P * P * P, NPL = (P3 + 31) / 32, G = kGroup;
    using SC = InferScratch<P>;
    extern __shared__ __align__(16) float smem_f[];
    float* sW = smem_f;                                   // [kParamsPad], W1 and W2 transposed
    float* sv = sW + kParamsPad + (threadIdx.x >> 5) * SC::per_warp;
    float* st = sv + SC::V;
    float* sx = st + SC::V;   // [64][G]
    float* sh = sx + 64 * G;  // [64][G]
    Scalars* s = dv.sc;
    if (!s->active) return;
    if (gated && s->sensor_fallback) return;
    {
        const float4* src = reinterpret_cast<const float4*>(Wt);
        float4* dst = reinterpret_cast<float4*>(sW);
        for (int i = threadIdx.x; i < kParamsPad / 4; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const float cut = fmaxf(f64_to_f32(bp.amin), kLearnedCut), amax = f64_to_f32(bp.amax);
    const float gm = f64_to_f32(g.gamma);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlock;
    int64_t cell = (int64_t)blockIdx.x * kWarpsPerBlock + warp;
    float u[NPL][5];
    if (cell < dv.nc) load_cell_f32<P, NPL>(dv, cell, lane, u);
    while (cell < dv.nc) {
        // G cells of this warp's sequence: inputs (and the plain indicator of handed-back cells)
        int64_t cg[G];
        float am[G];
        bool mk[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            cg[g] = cell;
            mk[g] = false;
            am[g] = 0.0f;
            if (cell < dv.nc) {
                float un[NPL][5];  // next cell's state, in flight during this cell's work
                if (cell + stride < dv.nc) load_cell_f32<P, NPL>(dv, cell + stride, lane, un);
                features_from_state<P, NPL, G>(dv, cell, gm, ip, u, sv, st, sx + g);
                if (mask && mask[cell]) {
                    mk[g] = true;
                    am[g] = modal_alpha_warp<P, NPL>(ops, bp, gm, u, sv, st);
                }
#pragma unroll
                for (int j = 0; j < NPL; ++j)
#pragma unroll
                    for (int v = 0; v < 5; ++v) u[j][v] = un[j][v];
            } else {
                sx[lane * G + g] = 0.0f;
                sx[(lane + 32) * G + g] = 0.0f;
                __syncwarp();
            }
            cell += stride;
        }
        float at[G];
        mlp_forward_group<G>(sW, sx, sh, amax, at);
        if (lane == 0) {
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (cg[g] >= dv.nc) continue;
                double a = mk[g] ? f32_to_f64(am[g]) : ((at[g] < cut) ? 0.0 : f32_to_f64(at[g]));
                if (dv.cell_wall[cg[g]]) {
                    const double wl = eval_expr(dv, bp.expr_wall, 0, 0, 0, s->time);
                    a = (wl > a) ? wl : a;
                }
                out[cg[g]] = a;
            }
        }
        __syncwarp();
    }
}

// The same inference with the two hidden layers on the tensor cores (mlp_tc.cuh), in two kernels:
// k_sensor_inputs computes every cell's network input at full occupancy and writes it, already
// split into TF32 hi/lo parts, in the shared-memory image of its 128-cell tile (the canonical
// operand layout: a tile is one contiguous 64 KB block); k_sensor_mlp_tc then moves a tile with
// one TMA bulk copy, runs each hidden layer as 24 tcgen05.mma, and every thread finishes its own
// row (bias, GELU, the output layer) from the accumulator in tensor memory.
constexpr int kTcParams = 4 * tc::kK * tc::kN + 3 * tc::kN + 4;  // W1 hi/lo, W2 hi/lo, b1, b2, w3, b3 (+pad)
constexpr int kTileFloats = 2 * tc::kRows * tc::kK;              // A hi + A lo of one tile

template <int P>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, (P <= 4 ? 3 : 1))
    k_sensor_inputs(Dev dv, GasP g, BlendP bp, Ops ops, Interp ip, float* __restrict__ tiles, float* __restrict__ mod,
                    int gated, const uint8_t* mask)
{
    constexpr int P3 = P * P * P, NPL = (P3 + 31) / 32;
    using SC = InferScratch<P>;
    extern __shared__ __align__(16) float smem_in[];
    float* sv = smem_in + (threadIdx.x >> 5) * (2 * SC::V + 64);
    float* st = sv + SC::V;
    float* sx = st + SC::V;
    Scalars* s = dv.sc;
    if (!s->active) return;
    if (gated && s->sensor_fallback) return;
    const float gm = f64_to_f32(g.gamma);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlock;
    int64_t cell = (int64_t)blockIdx.x * kWarpsPerBlock + warp;
    float u[NPL][5];
    if (cell < dv.nc) load_cell_f32<P, NPL>(dv, cell, lane, u);
    for (; cell < dv.nc; cell += stride) {
        float un[NPL][5];  // next cell's state, in flight during this cell's work
        if (cell + stride < dv.nc) load_cell_f32<P, NPL>(dv, cell + stride, lane, un);
        features_from_state<P, NPL, 1>(dv, cell, gm, ip, u, sv, st, sx);
        float am = -1.0f;
        if (mask && mask[cell]) am = modal_alpha_warp<P, NPL>(ops, bp, gm, u, sv, st);
        float* t = tiles + (cell / tc::kRows) * kTileFloats;
        const int row = (int)(cell % tc::kRows);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int k = lane + 32 * j;
            const float x = sx[k], hi = tc::tf32_hi(x);
            t[tc::core_off(row, k)] = hi;
            t[tc::kRows * tc::kK + tc::core_off(row, k)] = x - hi;
        }
        if (lane == 0) mod[cell] = am;
        __syncwarp();
#pragma unroll
        for (int j = 0; j < NPL; ++j)
#pragma unroll
            for (int v = 0; v < 5; ++v) u[j][v] = un[j][v];
    }
}

struct TcMlpSmem {
    static constexpr size_t oB = 0;                                  // W1 hi/lo, W2 hi/lo, biases
    static constexpr size_t oA = (kTcParams + 31) / 32 * 32;        // tile: A hi, A lo
    static constexpr size_t bytes = (oA + kTileFloats) * sizeof(float);
};

__global__ void __launch_bounds__(128, 1) k_sensor_mlp_tc(Dev dv, const float* __restrict__ Wtc,
                                                          const float* __restrict__ tiles,
                                                          const float* __restrict__ mod, BlendP bp, double* out,
                                                          int gated)
{
    extern __shared__ __align__(128) float smem_mlp[];
    __shared__ __align__(8) uint64_t bar_ld, bar_mma;
    __shared__ uint32_t tmem_base;
    float* sB = smem_mlp + TcMlpSmem::oB;
    float* sAhi = smem_mlp + TcMlpSmem::oA;
    float* sAlo = sAhi + tc::kRows * tc::kK;
    const float* W1hi = sB;
    const float* W1lo = sB + tc::kK * tc::kN;
    const float* W2hi = sB + 2 * tc::kK * tc::kN;
    const float* W2lo = sB + 3 * tc::kK * tc::kN;
    const float* b1 = sB + 4 * tc::kK * tc::kN;
    const float* b2 = b1 + 64;
    const float* w3 = b2 + 64;
    Scalars* s = dv.sc;
    if (!s->active) return;
    if (gated && s->sensor_fallback) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (dv.nc + tc::kRows - 1) / tc::kRows;
    if (warp == 0) tc::tmem_alloc(&tmem_base);
    if (tid == 0) {
        mbar_init(&bar_ld, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        int64_t t0 = blockIdx.x;
        mbar_arrive_expect_tx(&bar_ld, (uint32_t)(kTcParams * 4 + kTileFloats * 4));
        tma_load_1d(sB, Wtc, (uint32_t)(kTcParams * 4), &bar_ld);
        tma_load_1d(sAhi, tiles + t0 * kTileFloats, (uint32_t)(kTileFloats * 4), &bar_ld);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
    const int row = 32 * warp + lane;
    const float cut = fmaxf(f64_to_f32(bp.amin), kLearnedCut), amax = f64_to_f32(bp.amax);
    uint32_t ph_ld = 0, ph_mma = 0;
    bool ok = true;
    auto wait = [&](uint64_t* bar, uint32_t& ph) {
        bool done = false;
        for (int it = 0; it < (1 << 22) && !done; ++it) done = mbar_try_wait(bar, ph);
        ok = __syncthreads_and(done ? 1 : 0) != 0;
        if (ok) ph ^= 1;
    };
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        wait(&bar_ld, ph_ld);  // this tile's inputs (and, first, the weights) are in shared memory
        if (!ok) break;
        float v[2][32];
        // hidden layer 1: the accumulator, plus bias and GELU, becomes hidden layer 2's input
        if (tid == 0) {
            tc::fence_after();
            tc::layer_mma(tmem, sAhi, sAlo, W1hi, W1lo);
            tc::mma_commit(&bar_mma);
        }
        wait(&bar_mma, ph_mma);
        if (!ok) break;
        tc::fence_after();
        tc::tmem_ld32(taddr, v[0]);
        tc::tmem_ld32(taddr + 32, v[1]);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const int col = 32 * hh + i;
                const float x = gelu(v[hh][i] + b1[col]), hi = tc::tf32_hi(x);
                sAhi[tc::core_off(row, col)] = hi;
                sAlo[tc::core_off(row, col)] = x - hi;
            }
        tc::fence_smem_async();
        tc::fence_before();
        __syncthreads();
        // hidden layer 2
        if (tid == 0) {
            tc::fence_after();
            tc::layer_mma(tmem, sAhi, sAlo, W2hi, W2lo);
            tc::mma_commit(&bar_mma);
        }
        wait(&bar_mma, ph_mma);
        if (!ok) break;
        tc::fence_after();
        tc::tmem_ld32(taddr, v[0]);
        tc::tmem_ld32(taddr + 32, v[1]);
        float z = w3[64];  // b3 (the weights arrived with the first tile)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
            for (int i = 0; i < 32; ++i) z += w3[32 * hh + i] * gelu(v[hh][i] + b2[32 * hh + i]);
        const int64_t cell = tile * tc::kRows + row;
        if (cell < dv.nc) {
            const float at = amax / (1.0f + expf(-z)), am = mod[cell];
            double a = (am >= 0.0f) ? f32_to_f64(am) : ((at < cut) ? 0.0 : f32_to_f64(at));
            if (dv.cell_wall[cell]) {
                const double wl = eval_expr(dv, bp.expr_wall, 0, 0, 0, s->time);
                a = (wl > a) ? wl : a;
            }
            out[cell] = a;
        }
        tc::fence_before();
        __syncthreads();  // every row has read the accumulator and the tile buffer is free
        const int64_t next = tile + gridDim.x;
        if (tid == 0 && next < ntiles) {
            tc::fence_after();
            mbar_arrive_expect_tx(&bar_ld, (uint32_t)(kTileFloats * 4));
            tma_load_1d(sAhi, tiles + next * kTileFloats, (uint32_t)(kTileFloats * 4), &bar_ld);
        }
    }
    if (!ok) {
        if (tid == 0) s->err = PLENS_GPU_E_TIMEOUT;
        for (int it = 0; it < (1 << 22); ++it)  // copies and MMAs in flight complete first
            if (mbar_try_wait(&bar_ld, ph_ld)) break;
        for (int it = 0; it < (1 << 22); ++it)
            if (mbar_try_wait(&bar_mma, ph_mma)) break;
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem);
}

// judge (per cell, before smoothing): where |alpha_mlp - alpha_plain| exceeds the tolerance the
// plain value is kept and the cell is marked, so the plain indicator keeps computing it until the
// next judged step; elsewhere the MLP value is used. The smoothing max(a, a_nbr/2) is 1-Lipschitz
// in the max norm, so this bounds the error of the final alpha on judged steps.
__global__ void k_judge_cells(Dev dv, const double* alpha_mlp, uint8_t* mask, double tol,
                              unsigned long long* maxerr, unsigned int* nbad)
{
    if (!dv.sc->active) return;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double e = 0;
    unsigned int bad = 0;
    if (c < dv.nc) {
        e = fabs(alpha_mlp[c] - dv.alpha_raw[c]);
        bad = (e > tol) ? 1u : 0u;
        mask[c] = (uint8_t)bad;
        if (!bad) dv.alpha_raw[c] = alpha_mlp[c];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, e, off);
        e = (o > e) ? o : e;
        bad += __shfl_xor_sync(0xffffffffu, bad, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxerr, ord_double(e));
        if (bad) atomicAdd(nbad, bad);
    }
}

// judged-step bookkeeping; the whole domain falls back to the plain indicator when more than a
// tenth of the cells are over the tolerance
__global__ void k_judge_decide(Dev dv, unsigned long long* maxerr, unsigned int* nbad)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    const double e = unord_double(*maxerr);
    s->judged += 1;
    if (e > s->max_alpha_err) s->max_alpha_err = e;
    s->fallbacks += *nbad;
    s->sensor_fallback = (*nbad > (unsigned int)(dv.nc / 10)) ? 1 : 0;
    *maxerr = ord_double(0.0);
    *nbad = 0;
}

template <int P>
__global__ void k_features(Dev dv, GasP g, Interp ip, float* x)
{
    __shared__ float sv[kWarpsPerBlock][kMaxP * kMaxP * kMaxP];
    __shared__ float st[kWarpsPerBlock][4 * kMaxP * kMaxP];
    __shared__ float sx[kWarpsPerBlock][64];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t cell = (int64_t)blockIdx.x * kWarpsPerBlock + warp; cell < dv.nc; cell += (int64_t)gridDim.x * kWarpsPerBlock) {
        cell_features<P>(dv, g.gamma, ip, cell, sv[warp], st[warp], sx[warp]);
        x[cell * 64 + lane] = sx[warp][lane];
        x[cell * 64 + lane + 32] = sx[warp][lane + 32];
        __syncwarp();
    }
}

// The learned sensor at N = 3 in one kernel with the network and the judge's plain indicator on
// the tensor cores: one 128-cell tile per SM, 16 warps.
//  - The tile's FP32 state is staged in two halves of 64 cells (five bulk copies each); thread t
//    takes node t % 64 of cells 8 i + t / 64, forms rho*p with the positivity assertion, and the
//    cell's 64 values are normalised by their mean (the features of interp_normalise at P = 4,
//    where the interpolation to the 4^3 nodes is the identity).
//  - The features, split into TF32 hi/lo parts, are the A operand (K-major, K stride padded to 144
//    bytes: no bank conflicts); tcgen05.mma in 3xTF32 form computes layer 1 (B = W1) and, for the
//    cells the judge handed back, the change of basis of the features (B = C1 (x) C1 (x) C1; the
//    modal coefficients of rho*p are the mean times those plus C's row sums, and the indicator's
//    energy ratios do not depend on the mean).
//  - Warp w reads rows 32 (w % 4) .. + 31 and 16 columns 16 (w / 4) .. + 15 of each accumulator:
//    bias + GELU become layer 2's A operand, the modal energies are summed per cell; after layer 2
//    (B = W2) the warps sum their columns' share of the output layer; the first 128 threads
//    finish their cell: sigmoid x alpha_max, the cut, the plain indicator where the judge handed
//    the cell back, the wall override.
struct SensorTcSmem {
    static constexpr int kW = kTcParams;                        // W1 hi/lo, W2 hi/lo, b1, b2, w3, b3
    static constexpr int kC = 2 * 64 * 64 + 64;                 // C hi/lo and C's row sums
    static constexpr int kHalf = 5 * 64 * 64;                   // staged state of 64 cells (floats)
    static constexpr size_t oW = 0, oC = (kW + 31) / 32 * 32, oS = oC + (kC + 31) / 32 * 32;
    static constexpr int kOp = 2 * BtcSmem::kA;                 // an operand pair (hi, lo), padded layout
    static constexpr int kS = (kHalf > kOp ? kHalf : kOp);      // staging, then A, then H
    static constexpr size_t bytes = sizeof(float) * (oS + kS);
};

template <int P>
__global__ void __launch_bounds__(kBtcThreads, 1) k_sensor_tc(Dev dv, const float* __restrict__ Wtc,
                                                              const float* __restrict__ Ctc, BlendP bp, GasP g,
                                                              double* out, int gated, const uint8_t* mask, int tr)
{
    static_assert(P == 4, "the fused tensor-core sensor takes the 4^3 nodes of degree 3 as its inputs");
    constexpr int N = 3, P3 = 64, R = tc::kRows;
    extern __shared__ __align__(128) float smem_stc[];
    __shared__ __align__(8) uint64_t bar_ld, bar_mma;
    __shared__ uint32_t tmem_base;
    __shared__ float s_half[R][2], s_mean[R];
    __shared__ float s_e[4][3][R], s_z[4][R];
    float* sW = smem_stc + SensorTcSmem::oW;
    const float* W1hi = sW;
    const float* W1lo = sW + 4096;
    const float* W2hi = sW + 2 * 4096;
    const float* W2lo = sW + 3 * 4096;
    const float* b1 = sW + 4 * 4096;
    const float* b2 = b1 + 64;
    const float* w3 = b2 + 64;
    float* sC = smem_stc + SensorTcSmem::oC;
    const float* Chi = sC;
    const float* Clo = sC + 4096;
    const float* Crow = sC + 8192;
    float* sS = smem_stc + SensorTcSmem::oS;  // [5][64][64] staging, then A hi/lo, then H hi/lo
    float* sOhi = sS;
    float* sOlo = sS + BtcSmem::kA;
    Scalars* s = dv.sc;
    if (!s->active) return;
    // whole-domain fallback: every cell takes the plain indicator computed here
    const bool all_plain = gated && s->sensor_fallback;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (dv.nc + tr - 1) / tr;  // tiles of tr <= R cells
    const float gm = f64_to_f32(g.gamma);
    const float cut = fmaxf(f64_to_f32(bp.amin), kLearnedCut), amax = f64_to_f32(bp.amax);
    constexpr uint32_t kCols = 256;  // three 64-column accumulators
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::s_addr(&tmem_base)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bar_ld, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_base;
    uint32_t ph_ld = 0, ph_mma = 0;
    bool ok = true, first = true, mma_out = false;
    auto wait = [&](uint64_t* bar, uint32_t& ph) {
        bool done = false;
        for (int it = 0; it < (1 << 22) && !done; ++it) done = mbar_try_wait(bar, ph);
        ok = __syncthreads_and(done ? 1 : 0) != 0;
        if (ok) ph ^= 1;
    };
    const int node = tid & 63, q = warp & 3, cg = warp >> 2;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t c0 = tile * tr;
        const int ncell = (int)((dv.nc - c0 < tr) ? dv.nc - c0 : tr);
        float v[16];
        // ---- two halves of 64 cells: stage, rho*p, the per-cell sums
        for (int h = 0; h < 2 && ok; ++h) {
            const int nh = ncell - 64 * h < 64 ? (ncell - 64 * h > 0 ? ncell - 64 * h : 0) : 64;
            if (tid == 0) {
                const uint32_t bv = (uint32_t)(nh * P3 * 4);
                mbar_arrive_expect_tx(&bar_ld, 5 * bv + (first ? (uint32_t)(SensorTcSmem::kW * 4 + SensorTcSmem::kC * 4) : 0u));
                if (first) {
                    tma_load_1d(sW, Wtc, (uint32_t)(SensorTcSmem::kW * 4), &bar_ld);
                    tma_load_1d(sC, Ctc, (uint32_t)(SensorTcSmem::kC * 4), &bar_ld);
                }
                if (nh > 0)
#pragma unroll
                    for (int vv = 0; vv < 5; ++vv)
                        tma_load_1d(sS + vv * 64 * P3, dv.Uf + vv * dv.nd + (c0 + 64 * h) * P3, bv, &bar_ld);
            }
            first = false;
            wait(&bar_ld, ph_ld);
            if (!ok) break;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int rl = 8 * i + (tid >> 6), r = 64 * h + rl;  // local and tile row
                float val = 0.0f;
                if (r < ncell) {
                    float cf[5];
#pragma unroll
                    for (int vv = 0; vv < 5; ++vv) cf[vv] = sS[(vv * 64 + rl) * P3 + node];
                    const int64_t dof = (c0 + r) * P3 + node;
                    if (!positive_dof_screened(dv, dof, cf)) {
                        atomicMin(&s->bad_dof, (long long)dof);
                        s->err = PLENS_GPU_E_POSITIVITY;
                    }
                    val = get_p(cf, gm) * cf[0];
                }
                v[8 * h + i] = val;
                float sum = val;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                if (lane == 0) s_half[r][warp & 1] = sum;
            }
            __syncthreads();  // this half's staged values read
        }
        if (!ok) break;
        if (tid < R) s_mean[tid] = (s_half[tid][0] + s_half[tid][1]) * (1.0f / 64.0f);
        __syncthreads();
        // ---- features into the A operand
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int r = 8 * (i & 7) + (tid >> 6) + 64 * (i >> 3), o = a_off_padded(r, node);
            const float x = (r < ncell) ? v[i] * (1.0f / s_mean[r]) - 1.0f : 0.0f;
            const float hi = tc::tf32_hi(x);
            sOhi[o] = hi;
            sOlo[o] = x - hi;
        }
        tc::fence_smem_async();
        tc::fence_before();
        __syncthreads();
        // ---- layer 1 into columns 0..63, the change of basis into 64..127
        if (tid == 0) {
            tc::fence_after();
            cbm_mma(tmem, sOhi, sOlo, W1hi, W1lo);
            cbm_mma(tmem + 64, sOhi, sOlo, Chi, Clo);
            tc::mma_commit(&bar_mma);
        }
        mma_out = true;
        wait(&bar_mma, ph_mma);
        if (!ok) break;
        mma_out = false;
        tc::fence_after();
        {
            const int row = 32 * q + lane;
            const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16);
            float d[16];
            tc::tmem_ld16(ta + (uint32_t)(16 * cg), d);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float hv[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) hv[e] = gelu(d[4 * j + e] + b1[16 * cg + 4 * j + e]);
                const float4 hi = make_float4(tc::tf32_hi(hv[0]), tc::tf32_hi(hv[1]), tc::tf32_hi(hv[2]), tc::tf32_hi(hv[3]));
                const float4 lo = make_float4(hv[0] - hi.x, hv[1] - hi.y, hv[2] - hi.z, hv[3] - hi.w);
                const int o = a_off_padded(row, 16 * cg + 4 * j);
                *reinterpret_cast<float4*>(sOhi + o) = hi;
                *reinterpret_cast<float4*>(sOlo + o) = lo;
            }
            tc::tmem_ld16(ta + (uint32_t)(64 + 16 * cg), d);
            float e0 = 0, e1 = 0, e2 = 0;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int n = 16 * cg + i, mi = n % P, mj = (n / P) % P, mk = n / (P * P);
                const float md = d[i] + Crow[n], e = md * md;
                e0 += e;
                if (mi < N && mj < N && mk < N) e1 += e;
                if (mi < N - 1 && mj < N - 1 && mk < N - 1) e2 += e;
            }
            s_e[cg][0][row] = e0;
            s_e[cg][1][row] = e1;
            s_e[cg][2][row] = e2;
        }
        tc::fence_smem_async();
        tc::fence_before();
        __syncthreads();
        // ---- layer 2 into columns 128..191
        if (tid == 0) {
            tc::fence_after();
            cbm_mma(tmem + 128, sOhi, sOlo, W2hi, W2lo);
            tc::mma_commit(&bar_mma);
        }
        mma_out = true;
        wait(&bar_mma, ph_mma);
        if (!ok) break;
        mma_out = false;
        tc::fence_after();
        {
            const int row = 32 * q + lane;
            float d[16];
            tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(128 + 16 * cg), d);
            float z = 0.0f;
#pragma unroll
            for (int i = 0; i < 16; ++i) z += w3[16 * cg + i] * gelu(d[i] + b2[16 * cg + i]);
            s_z[cg][row] = z;
        }
        __syncthreads();
        if (tid < ncell) {
            const int64_t cell = c0 + tid;
            const float z = w3[64] + s_z[0][tid] + s_z[1][tid] + s_z[2][tid] + s_z[3][tid];
            const float at = amax / (1.0f + expf(-z));
            double a = (at < cut) ? 0.0 : f32_to_f64(at);
            if (all_plain || (mask && mask[cell])) {
                // the judge handed the cell back (or the whole domain is in fallback): the plain
                // modal indicator (FP32)
                const float e0 = s_e[0][0][tid] + s_e[1][0][tid] + s_e[2][0][tid] + s_e[3][0][tid];
                const float e1 = s_e[0][1][tid] + s_e[1][1][tid] + s_e[2][1][tid] + s_e[3][1][tid];
                const float e2 = s_e[0][2][tid] + s_e[1][2][tid] + s_e[2][2][tid] + s_e[3][2][tid];
                float trouble = 1.0f - __fdividef(e1, e0);
                const float t2 = 1.0f - __fdividef(e2, e1);
                if (t2 > trouble) trouble = t2;
                const float thr = f64_to_f32(bp.thr), amin = f64_to_f32(bp.amin);
                float alpha;
                if (bp.func == 0) {
                    const float ah = __fdividef(1.0f, 1.0f + __expf(-f64_to_f32(bp.sharp) * (__fdividef(trouble, thr) - 1.0f)));
                    alpha = (ah < amin) ? 0.0f : (ah < amax ? ah : amax);
                } else {
                    const float ah = __fdividef(trouble, thr);
                    alpha = (ah > 1.0f) ? 1.0f : ah;
                }
                a = f32_to_f64(alpha);
            }
            if (dv.cell_wall[cell]) {
                const double wl = eval_expr(dv, bp.expr_wall, 0, 0, 0, s->time);
                a = (wl > a) ? wl : a;
            }
            out[cell] = a;
        }
        tc::fence_before();
        __syncthreads();  // accumulators read, shared operands free for the next tile
        tc::fence_after();
    }
    if (!ok) {
        if (tid == 0) s->err = PLENS_GPU_E_TIMEOUT;
        for (int it = 0; it < (1 << 22) && !mbar_try_wait(&bar_ld, ph_ld); ++it) {
        }
        if (mma_out)
            for (int it = 0; it < (1 << 22) && !mbar_try_wait(&bar_mma, ph_mma); ++it) {
            }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
}

// the fused tensor-core sensor (degree 3 only; 0 launches otherwise)
template <int P>
int launch_sensor_tc(MlpDevice& m, const Dev& dv, const GasP& g, const BlendP& bp, double* out, int gated,
                     const uint8_t* mask, cudaStream_t st)
{
    if constexpr (P == 4) {
        static int nsm = 0;
        if (!nsm) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaFuncSetAttribute(k_sensor_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SensorTcSmem::bytes);
            nsm = std::max(1, nsm);
        }
        const int tr = tc::tile_rows(dv.nc, nsm);
        const int64_t tiles = (dv.nc + tr - 1) / tr;
        k_sensor_tc<P><<<(unsigned)std::min<int64_t>(tiles, nsm), kBtcThreads, SensorTcSmem::bytes, st>>>(
            dv, m.params_tc, m.cbm, bp, g, out, gated, mask, tr);
        return 1;
    } else {
        return 0;
    }
}

template <int P>
int launch_infer_tc(MlpDevice& m, const Dev& dv, const GasP& g, const BlendP& bp, const Ops& ops, double* out,
                    int gated, const uint8_t* mask, cudaStream_t st)
{
    const Interp ip = make_interp(P);
    const size_t in_bytes = sizeof(float) * kWarpsPerBlock * (2 * InferScratch<P>::V + 64);
    static int in_blocks = 0, nsm = 0;
    if (!in_blocks) {
        cudaFuncSetAttribute(k_sensor_inputs<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)in_bytes);
        int dev = 0, occ = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sensor_inputs<P>, 32 * kWarpsPerBlock, in_bytes);
        nsm = std::max(1, nsm);
        in_blocks = std::max(1, occ) * nsm;
        cudaFuncSetAttribute(k_sensor_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TcMlpSmem::bytes);
    }
    const int64_t tiles = (dv.nc + tc::kRows - 1) / tc::kRows;
    if (tiles < 1) return 0;
    const int64_t blocks = std::min<int64_t>((dv.nc + kWarpsPerBlock - 1) / kWarpsPerBlock, in_blocks);
    k_sensor_inputs<P><<<(unsigned)blocks, 32 * kWarpsPerBlock, in_bytes, st>>>(dv, g, bp, ops, ip, m.tiles, m.mod,
                                                                             gated, mask);
    k_sensor_mlp_tc<<<(unsigned)std::min<int64_t>(tiles, nsm), 128, TcMlpSmem::bytes, st>>>(dv, m.params_tc, m.tiles,
                                                                                         m.mod, bp, out, gated);
    return 2;
}

template <int P>
int launch_infer(const Dev& dv, const float* Wt, const GasP& g, const BlendP& bp, const Ops& ops, double* out,
                 int gated, const uint8_t* mask, cudaStream_t st)
{
    const Interp ip = make_interp(P);
    const size_t bytes = sizeof(float) * (kParamsPad + kWarpsPerBlock * InferScratch<P>::per_warp);
    static int per_sm = 0;
    if (!per_sm) {
        cudaFuncSetAttribute(k_sensor_infer<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sensor_infer<P>, 32 * kWarpsPerBlock, bytes);
        per_sm = std::max(1, occ) * std::max(1, nsm);
    }
    const int64_t blocks = std::min<int64_t>((dv.nc + kWarpsPerBlock - 1) / kWarpsPerBlock, per_sm);
    k_sensor_infer<P><<<(unsigned)blocks, 32 * kWarpsPerBlock, bytes, st>>>(dv, Wt, g, bp, ops, ip, out, gated, mask);
    return 1;
}

// plain indicator (FP64, the judge) on every cell; `limit` caps the grid (the block loop covers
// the rest) for the launch that only runs in whole-domain fallback
template <int P>
int launch_blender(const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, cudaStream_t st, int64_t limit = 0)
{
    using CB = CellBlock<P>;
    int64_t blocks = (dv.nc + CB::CPB - 1) / CB::CPB;
    if (limit > 0 && blocks > limit) blocks = limit;
    k_blender<P, double><<<(unsigned)blocks, CB::THREADS, 0, st>>>(dv, ops, g, bp);
    return 1;
}

// One stage's blender with the learned sensor. Non-judged stages: the MLP into alpha_raw for
// every cell (skipped in whole-domain fallback), then the plain modal indicator for the cells the
// last judge handed back (all cells in fallback), then the neighbour smoothing + alpha_d +
// compacted troubled-cell list. Judged stage (stage 1 of every judge_every-th step): MLP and
// plain indicator for all cells, per-cell comparison and takeover.
template <int P>
int sensor_stage(MlpDevice& m, const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, cudaStream_t st)
{
    int n = 0;
    BlendP b0 = bp;
    b0.gate = 0;
    b0.mask = nullptr;
    // degree 3 with the network on the tensor cores: the fused kernel (its plain indicator for
    // handed-back cells takes the change of basis of the rho*p features: the default indicator
    // variable)
    const bool fused_tc = P == 4 && m.use_tc && m.cbm && bp.var == 0;
    if (m.judge_this_step) {
        n += fused_tc ? launch_sensor_tc<P>(m, dv, g, bp, m.alpha_plain, 0, nullptr, st)
             : m.use_tc ? launch_infer_tc<P>(m, dv, g, bp, ops, m.alpha_plain, 0, nullptr, st)
                        : launch_infer<P>(dv, m.params_t, g, bp, ops, m.alpha_plain, 0, nullptr, st);
        n += launch_blender<P>(dv, ops, g, b0, st);
        const unsigned grid = (unsigned)((dv.nc + 127) / 128);
        k_judge_cells<<<grid, 128, 0, st>>>(dv, m.alpha_plain, m.mask, m.tol, m.maxerr, m.nbad);
        k_judge_decide<<<1, 1, 0, st>>>(dv, m.maxerr, m.nbad);
        n += 2;
        m.judge_this_step = false;  // the remaining stages of this step follow the decision
    } else {
        // the cells the judge handed back get the plain indicator inside the inference kernel;
        // in whole-domain fallback the plain blender runs instead (the fused tensor-core kernel
        // computes the plain indicator of every cell then itself)
        n += fused_tc ? launch_sensor_tc<P>(m, dv, g, bp, dv.alpha_raw, 1, m.mask, st)
             : m.use_tc ? launch_infer_tc<P>(m, dv, g, bp, ops, dv.alpha_raw, 1, m.mask, st)
                        : launch_infer<P>(dv, m.params_t, g, bp, ops, dv.alpha_raw, 1, m.mask, st);
        if (!fused_tc) {
            BlendP b1 = bp;
            b1.gate = 1;
            b1.mask = nullptr;
            n += launch_blender<P>(dv, ops, g, b1, st, 152 * 2);
        }
    }
    k_alpha_smooth<<<(unsigned)((dv.nc + kSmoothThreads - 1) / kSmoothThreads), kSmoothThreads, 0, st>>>(dv, b0);
    return n + 1;
}

}  // namespace

int mlp_create(MlpDevice& m, int64_t nc, std::vector<void*>& allocs)
{
    m.nc = nc;
    if (cudaMalloc(&m.params, sizeof(float) * kMlpParams) != cudaSuccess) return 1;
    allocs.push_back(m.params);
    if (cudaMalloc(&m.params_t, sizeof(float) * kParamsPad) != cudaSuccess) return 1;
    allocs.push_back(m.params_t);
    if (cudaMalloc(&m.params_tc, sizeof(float) * kTcParams) != cudaSuccess) return 1;
    allocs.push_back(m.params_tc);
    {
        // network inputs in tile images (rows past the last cell stay zero) and the plain
        // indicator of handed-back cells
        const int64_t ntiles = (nc + tc::kRows - 1) / tc::kRows;
        if (cudaMalloc(&m.tiles, sizeof(float) * kTileFloats * ntiles) != cudaSuccess ||
            cudaMemset(m.tiles, 0, sizeof(float) * kTileFloats * ntiles) != cudaSuccess)
            return 1;
        allocs.push_back(m.tiles);
        if (cudaMalloc(&m.mod, sizeof(float) * nc) != cudaSuccess) return 1;
        allocs.push_back(m.mod);
    }
    if (cudaMalloc(&m.alpha_plain, sizeof(double) * (nc + 1)) != cudaSuccess) return 1;
    allocs.push_back(m.alpha_plain);
    if (cudaMalloc(&m.maxerr, sizeof(unsigned long long)) != cudaSuccess) return 1;
    allocs.push_back(m.maxerr);
    if (cudaMalloc(&m.mask, nc) != cudaSuccess || cudaMemset(m.mask, 0, nc) != cudaSuccess) return 1;
    allocs.push_back(m.mask);
    if (cudaMalloc(&m.nbad, sizeof(unsigned int)) != cudaSuccess || cudaMemset(m.nbad, 0, sizeof(unsigned int)) != cudaSuccess) return 1;
    allocs.push_back(m.nbad);
    const unsigned long long z = ord_double_host(0.0);
    if (cudaMemcpy(m.maxerr, &z, sizeof(z), cudaMemcpyHostToDevice) != cudaSuccess) return 1;
    return 0;
}

int mlp_set_weights(MlpDevice& m, const float* host_params, cudaStream_t st)
{
    // the inference kernel's copy: W1 and W2 transposed ([in][out]), padded to float4s
    std::vector<float> t(kParamsPad, 0.0f);
    for (int i = 0; i < kMlpParams; ++i) {
        int dst = i;
        if (i < kMlpHid * kMlpIn) {
            const int o = i / kMlpIn, k = i - o * kMlpIn;
            dst = k * kMlpHid + o;
        } else {
            const int base = kMlpHid * kMlpIn + kMlpHid;
            if (i >= base && i < base + kMlpHid * kMlpHid) {
                const int r = i - base, o = r / kMlpHid, k = r - o * kMlpHid;
                dst = base + k * kMlpHid + o;
            }
        }
        t[dst] = host_params[i];
    }
    // the tensor-core copy: W1 and W2 ([out][in], i.e. the B operands N x K) split into TF32 hi
    // and lo parts in the canonical operand layout, then b1, b2, w3, b3
    std::vector<float> w(kTcParams, 0.0f);
    {
        const float* W1 = host_params;
        const float* B1 = W1 + kMlpHid * kMlpIn;
        const float* W2 = B1 + kMlpHid;
        const float* B2 = W2 + kMlpHid * kMlpHid;
        const float* W3 = B2 + kMlpHid;
        const int mat = tc::kK * tc::kN;
        for (int o = 0; o < kMlpHid; ++o)
            for (int k = 0; k < kMlpIn; ++k) {
                const int off = tc::core_off(o, k);
                const float a = W1[o * kMlpIn + k], b = W2[o * kMlpHid + k];
                const float ah = tc::tf32_hi(a), bh = tc::tf32_hi(b);
                w[off] = ah;
                w[mat + off] = a - ah;
                w[2 * mat + off] = bh;
                w[3 * mat + off] = b - bh;
            }
        for (int i = 0; i < kMlpHid; ++i) {
            w[4 * mat + i] = B1[i];
            w[4 * mat + 64 + i] = B2[i];
            w[4 * mat + 128 + i] = W3[i];
        }
        w[4 * mat + 192] = W3[kMlpHid];
    }
    if (cudaMemcpyAsync(m.params_tc, w.data(), sizeof(float) * kTcParams, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return 1;
    if (cudaMemcpyAsync(m.params, host_params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, st) != cudaSuccess) return 1;
    if (cudaMemcpyAsync(m.params_t, t.data(), sizeof(float) * kParamsPad, cudaMemcpyHostToDevice, st) != cudaSuccess) return 1;
    if (cudaStreamSynchronize(st) != cudaSuccess) return 1;
    m.weights_set = true;
    return 0;
}

int mlp_sensor_launch(MlpDevice& m, const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, int P,
                      cudaStream_t st)
{
    switch (P) {
    case 2: return sensor_stage<2>(m, dv, ops, g, bp, st);
    case 3: return sensor_stage<3>(m, dv, ops, g, bp, st);
    case 4: return sensor_stage<4>(m, dv, ops, g, bp, st);
    case 5: return sensor_stage<5>(m, dv, ops, g, bp, st);
    default: return sensor_stage<6>(m, dv, ops, g, bp, st);
    }
}

int mlp_step_begin(MlpDevice& m, const Dev& dv, int judge_every, cudaStream_t st)
{
    (void)dv;
    (void)st;
    m.judge_this_step = (judge_every <= 1) || (m.step_counter % judge_every == 0);
    ++m.step_counter;
    return 0;
}

int mlp_step_end(MlpDevice& m, const Dev& dv, cudaStream_t st)
{
    (void)m;
    (void)dv;
    (void)st;
    return 0;
}

int mlp_pairs(const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, int P, float* x, float* y,
              cudaStream_t st, int64_t& launches)
{
    float* dx = nullptr;
    if (cudaMalloc(&dx, sizeof(float) * 64 * dv.nc) != cudaSuccess) return PLENS_GPU_E_CUDA;
    k_step_begin<<<1, 1, 0, st>>>(dv, 1e300);
    BlendP b0 = bp;
    b0.gate = 0;
    const int64_t blocks = std::min<int64_t>((dv.nc + kWarpsPerBlock - 1) / kWarpsPerBlock, 152 * 8);
    switch (P) {
    case 2: launch_blender<2>(dv, ops, g, b0, st); k_features<2><<<(unsigned)blocks, 256, 0, st>>>(dv, g, make_interp(2), dx); break;
    case 3: launch_blender<3>(dv, ops, g, b0, st); k_features<3><<<(unsigned)blocks, 256, 0, st>>>(dv, g, make_interp(3), dx); break;
    case 4: launch_blender<4>(dv, ops, g, b0, st); k_features<4><<<(unsigned)blocks, 256, 0, st>>>(dv, g, make_interp(4), dx); break;
    case 5: launch_blender<5>(dv, ops, g, b0, st); k_features<5><<<(unsigned)blocks, 256, 0, st>>>(dv, g, make_interp(5), dx); break;
    default: launch_blender<6>(dv, ops, g, b0, st); k_features<6><<<(unsigned)blocks, 256, 0, st>>>(dv, g, make_interp(6), dx); break;
    }
    launches += 3;
    std::vector<double> a(dv.nc);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpy(x, dx, sizeof(float) * 64 * dv.nc, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(a.data(), dv.alpha_raw, sizeof(double) * dv.nc, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    if (e != cudaSuccess) return PLENS_GPU_E_CUDA;
    for (int64_t i = 0; i < dv.nc; ++i) y[i] = (float)a[i];
    return 0;
}

// ===================================================================== training kernels

namespace {

// a = act(x W^T + b) for a batch: one thread per (sample, output)
__global__ void k_dense_fwd(const float* __restrict__ X, int in, const float* __restrict__ W, const float* __restrict__ b,
                            int out, int64_t B, float* __restrict__ Apre, float* __restrict__ H)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= B * out) return;
    const int64_t s = i / out;
    const int o = (int)(i - s * out);
    float acc = b[o];
    for (int k = 0; k < in; ++k) acc += W[o * in + k] * X[s * in + k];
    Apre[i] = acc;
    H[i] = gelu(acc);
}

// output layer, loss and its gradient with respect to z
__global__ void k_head(const float* __restrict__ H2, const float* __restrict__ w3, float b3, const float* __restrict__ y,
                       int64_t B, float amax, float* __restrict__ alpha, float* __restrict__ dz, float* __restrict__ loss_terms)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= B) return;
    float z = b3;
    for (int k = 0; k < kMlpHid; ++k) z += w3[k] * H2[s * kMlpHid + k];
    const float sg = 1.0f / (1.0f + expf(-z));
    const float a = amax * sg;
    alpha[s] = a;
    if (y) {
        const float d = a - y[s];
        loss_terms[s] = d * d;
        dz[s] = (2.0f / (float)B) * d * amax * sg * (1.0f - sg);
    }
}

// dH_in[s][k] = sum_o dA[s][o] W[o][k], then times act'(Apre_in)
__global__ void k_dense_bwd_input(const float* __restrict__ dA, const float* __restrict__ W, int in, int out, int64_t B,
                                  const float* __restrict__ Apre_in, float* __restrict__ dA_in)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= B * in) return;
    const int64_t s = i / in;
    const int k = (int)(i - s * in);
    float acc = 0;
    for (int o = 0; o < out; ++o) acc += dA[s * out + o] * W[o * in + k];
    dA_in[i] = acc * gelu_d(Apre_in[i]);
}

// dW[o][k] = sum_s dA[s][o] X[s][k], db[o] = sum_s dA[s][o] (fixed summation order)
__global__ void k_dense_bwd_weight(const float* __restrict__ dA, const float* __restrict__ X, int in, int out, int64_t B,
                                   float* __restrict__ dW, float* __restrict__ db)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= out * (in + 1)) return;
    const int o = i / (in + 1), k = i - o * (in + 1);
    float acc = 0;
    if (k < in) {
        for (int64_t s = 0; s < B; ++s) acc += dA[s * out + o] * X[s * in + k];
        dW[o * in + k] = acc;
    } else {
        for (int64_t s = 0; s < B; ++s) acc += dA[s * out + o];
        db[o] = acc;
    }
}

// head gradients: dw3[k] = sum_s dz[s] H2[s][k], db3 = sum dz, dA2[s][k] = dz[s] w3[k] act'(A2)
__global__ void k_head_bwd(const float* __restrict__ dz, const float* __restrict__ H2, const float* __restrict__ A2,
                           const float* __restrict__ w3, int64_t B, float* __restrict__ dw3, float* __restrict__ db3,
                           float* __restrict__ dA2)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < B * kMlpHid) {
        const int64_t s = i / kMlpHid;
        const int k = (int)(i - s * kMlpHid);
        dA2[i] = dz[s] * w3[k] * gelu_d(A2[i]);
    }
    if (i < kMlpHid + 1) {
        float acc = 0;
        if (i < kMlpHid) {
            for (int64_t s = 0; s < B; ++s) acc += dz[s] * H2[s * kMlpHid + i];
            dw3[i] = acc;
        } else {
            for (int64_t s = 0; s < B; ++s) acc += dz[s];
            db3[0] = acc;
        }
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1 - b1) * gi;
    const float vi = b2 * v[i] + (1 - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_gather(const float* __restrict__ X, const float* __restrict__ Y, const int64_t* __restrict__ idx,
                         int64_t B, float* __restrict__ Xb, float* __restrict__ Yb)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= B * kMlpIn) return;
    const int64_t s = i / kMlpIn;
    const int k = (int)(i - s * kMlpIn);
    const int64_t src = idx[s];
    Xb[i] = X[src * kMlpIn + k];
    if (k == 0) Yb[s] = Y[src];
}

struct Trainer {
    int64_t cap = 0;
    float *x = nullptr, *y = nullptr, *a1 = nullptr, *h1 = nullptr, *a2 = nullptr, *h2 = nullptr;
    float *alpha = nullptr, *dz = nullptr, *lt = nullptr, *da2 = nullptr, *da1 = nullptr;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    cudaStream_t st = nullptr;
    std::vector<void*> allocs;
    bool ok = true;
    template <class T>
    void alloc(T** ptr, size_t n)
    {
        if (cudaMalloc(ptr, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) ok = false;
        else allocs.push_back(*ptr);
    }
    explicit Trainer(int64_t B) : cap(B)
    {
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        alloc(&x, B * kMlpIn); alloc(&y, B); alloc(&a1, B * kMlpHid); alloc(&h1, B * kMlpHid);
        alloc(&a2, B * kMlpHid); alloc(&h2, B * kMlpHid); alloc(&alpha, B); alloc(&dz, B); alloc(&lt, B);
        alloc(&da2, B * kMlpHid); alloc(&da1, B * kMlpHid);
        alloc(&p, kMlpParams); alloc(&g, kMlpParams); alloc(&m, kMlpParams); alloc(&v, kMlpParams);
    }
    ~Trainer()
    {
        if (st) cudaStreamSynchronize(st);
        for (void* q : allocs) cudaFree(q);
        if (st) cudaStreamDestroy(st);
    }
    // forward (+ backward when y given) of B samples already in x / y
    void run(int64_t B, float amax, bool backward)
    {
        const float* W1 = p;
        const float* b1 = W1 + kMlpHid * kMlpIn;
        const float* W2 = b1 + kMlpHid;
        const float* b2 = W2 + kMlpHid * kMlpHid;
        const float* w3 = b2 + kMlpHid;
        const unsigned gh = (unsigned)((B * kMlpHid + 255) / 256), gb = (unsigned)((B + 255) / 256);
        k_dense_fwd<<<gh, 256, 0, st>>>(x, kMlpIn, W1, b1, kMlpHid, B, a1, h1);
        k_dense_fwd<<<gh, 256, 0, st>>>(h1, kMlpHid, W2, b2, kMlpHid, B, a2, h2);
        float b3h;
        cudaMemcpyAsync(&b3h, w3 + kMlpHid, sizeof(float), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        k_head<<<gb, 256, 0, st>>>(h2, w3, b3h, backward ? y : nullptr, B, amax, alpha, dz, lt);
        if (!backward) return;
        float* gW1 = g;
        float* gb1 = gW1 + kMlpHid * kMlpIn;
        float* gW2 = gb1 + kMlpHid;
        float* gb2 = gW2 + kMlpHid * kMlpHid;
        float* gw3 = gb2 + kMlpHid;
        k_head_bwd<<<gh, 256, 0, st>>>(dz, h2, a2, w3, B, gw3, gw3 + kMlpHid, da2);
        k_dense_bwd_weight<<<(kMlpHid * (kMlpHid + 1) + 127) / 128, 128, 0, st>>>(da2, h1, kMlpHid, kMlpHid, B, gW2, gb2);
        k_dense_bwd_input<<<gh, 256, 0, st>>>(da2, W2, kMlpHid, kMlpHid, B, a1, da1);
        k_dense_bwd_weight<<<(kMlpHid * (kMlpIn + 1) + 127) / 128, 128, 0, st>>>(da1, x, kMlpIn, kMlpHid, B, gW1, gb1);
    }
    double loss(int64_t B)
    {
        std::vector<float> h(B);
        cudaMemcpyAsync(h.data(), lt, sizeof(float) * B, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        double s = 0;
        for (float t : h) s += t;
        return s / (double)B;
    }
};

}  // namespace

}  // namespace plens_gpu

using namespace plens_gpu;

extern "C" {

int plens_gpu_mlp_loss_grad(const float* x, const float* y, int64_t n, const float* params, float alpha_max,
                            float* loss, float* grad)
{
    if (!x || !y || !params || n <= 0) return PLENS_GPU_E_INVALID;
    Trainer t(n);
    if (!t.ok) return PLENS_GPU_E_CUDA;
    cudaMemcpy(t.x, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice);
    cudaMemcpy(t.y, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(t.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    t.run(n, alpha_max, true);
    if (loss) *loss = (float)t.loss(n);
    if (grad) cudaMemcpy(grad, t.g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost);
    return cudaGetLastError() == cudaSuccess ? 0 : PLENS_GPU_E_CUDA;
}

int plens_gpu_mlp_infer(const float* x, int64_t n, const float* params, float alpha_max, float* alpha)
{
    if (!x || !params || !alpha || n <= 0) return PLENS_GPU_E_INVALID;
    Trainer t(n);
    if (!t.ok) return PLENS_GPU_E_CUDA;
    cudaMemcpy(t.x, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice);
    cudaMemcpy(t.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    t.run(n, alpha_max, false);
    cudaStreamSynchronize(t.st);
    cudaMemcpy(alpha, t.alpha, sizeof(float) * n, cudaMemcpyDeviceToHost);
    return cudaGetLastError() == cudaSuccess ? 0 : PLENS_GPU_E_CUDA;
}

int plens_gpu_mlp_train(const float* x, const float* y, int64_t n, float* params, int32_t epochs, int32_t batch,
                        float lr, float alpha_max, uint64_t seed, float* loss_out)
{
    if (!x || !y || !params || n <= 0 || epochs < 0 || batch <= 0) return PLENS_GPU_E_INVALID;
    const int64_t B = std::min<int64_t>(batch, n);
    Trainer t(B);
    if (!t.ok) return PLENS_GPU_E_CUDA;
    float *dX = nullptr, *dY = nullptr;
    int64_t* dIdx = nullptr;
    if (cudaMalloc(&dX, sizeof(float) * n * kMlpIn) != cudaSuccess) return PLENS_GPU_E_CUDA;
    cudaMalloc(&dY, sizeof(float) * n);
    cudaMalloc(&dIdx, sizeof(int64_t) * n);
    cudaMemcpy(dX, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice);
    cudaMemcpy(dY, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(t.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    cudaMemset(t.m, 0, sizeof(float) * kMlpParams);
    cudaMemset(t.v, 0, sizeof(float) * kMlpParams);
    std::vector<int64_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::mt19937_64 rng(seed);
    int64_t step = 0;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(perm.begin(), perm.end(), rng);
        cudaMemcpyAsync(dIdx, perm.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, t.st);
        double ls = 0;
        int64_t seen = 0;
        for (int64_t off = 0; off < n; off += B) {
            const int64_t bsz = std::min<int64_t>(B, n - off);
            k_gather<<<(unsigned)((bsz * kMlpIn + 255) / 256), 256, 0, t.st>>>(dX, dY, dIdx + off, bsz, t.x, t.y);
            t.run(bsz, alpha_max, true);
            ++step;
            const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
            k_adam<<<(kMlpParams + 255) / 256, 256, 0, t.st>>>(t.p, t.g, t.m, t.v, kMlpParams, lr, b1, b2, eps, c1, c2);
            ls += t.loss(bsz) * (double)bsz;
            seen += bsz;
        }
        if (loss_out) loss_out[ep] = (float)(ls / (double)seen);
    }
    cudaStreamSynchronize(t.st);
    cudaMemcpy(params, t.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost);
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dIdx);
    return cudaGetLastError() == cudaSuccess ? 0 : PLENS_GPU_E_CUDA;
}

}  // extern "C"
