// blender_tc.cuh -- the modal troubled-cell indicator of the mixed forms at N = 3 with the change
// of basis on the 5th-generation tensor cores.
//
// BlenderCalculator::get_blender (dgsem/blender_calculator.cc:123-177) maps a cell's nodal values
// of the indicator variable (rho*p by default) to Legendre modal coefficients with the change of
// basis matrix (dgsem/change_of_basis_matrix.h:74-98), sums mode energies and turns them into
// alpha. For 128 cells at a time that is one [128 x 64] . [64 x 64]^T product: A holds the cells'
// nodal values (K-major, the canonical no-swizzle layout of mlp_tc.cuh), B the 64 x 64 matrix
// C = C1 (x) C1 (x) C1 (B[mode][node]), both split into TF32 hi/lo parts (3xTF32, FP32
// accumulation in tensor memory: 24 tcgen05.mma of K = 8, issued by one thread).
//
// Staging: one thread issues five bulk copies per tile (the tile's 128 cells x 64 nodes of each
// FP32 state variable are one contiguous 32 KB run). The block has 16 warps (latency hiding:
// one block per SM); thread t takes the nodes t % 64 of the cells 8 i + t / 64 (i = 0..15): a
// warp reads 32 consecutive floats (no bank conflicts), forms rho*p with the positivity
// assertion and keeps its 16 values in registers. A overlays the staging; its core matrices are
// laid out K-major with their K-direction stride (the descriptor's leading byte offset) padded
// from 128 to 144 bytes, so a warp's 32 consecutive nodes of one cell land in 32 different
// banks. Epilogue: warp w reads rows 32 (w % 4) .. + 31 (its lane quarter of tensor memory) and
// the 16 modes 16 (w / 4) .. + 15 (tcgen05.ld), sums their energies per cell; the four partial
// sums of a cell meet in shared memory and the first four warps form alpha as the CUDA-core
// kernel does (sums in mode order instead of a warp reduction).
#pragma once

#include "async.cuh"
#include "kernels.cuh"
#include "mlp_tc.cuh"

namespace plens_gpu {

struct BtcSmem {
    static constexpr int kB = 2 * 64 * 64;                   // B hi, B lo (floats), canonical layout
    static constexpr int kStage = 5 * tc::kRows * 64;        // staged state (floats)
    static constexpr int kLboA = 144, kSboA = 16 * kLboA;    // A's core-matrix strides (bytes)
    static constexpr int kA = tc::kRows / 8 * kSboA / 4;     // one A operand (floats)
    static constexpr size_t oB = 0, oS = kB;                 // float offsets; A hi/lo overlay oS
    static constexpr size_t bytes = sizeof(float) * (kB + kStage);
    static_assert(2 * kA <= kStage, "A hi/lo must fit in the staging area");
};

// float offset of A element (row r, k) with the padded K stride
__device__ __forceinline__ int a_off_padded(int r, int k)
{
    return (r >> 3) * (BtcSmem::kSboA / 4) + (k >> 2) * (BtcSmem::kLboA / 4) + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ uint64_t desc_kmajor_padded(const void* p)
{
    const uint32_t a = tc::s_addr(p);
    uint64_t d = (uint64_t)((a >> 4) & 0x3FFFu);
    d |= (uint64_t)(BtcSmem::kLboA >> 4) << 16;
    d |= (uint64_t)(BtcSmem::kSboA >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// D = A x B^T in 3xTF32 (24 MMAs of K = 8): A with the padded strides, B canonical
__device__ __forceinline__ void cbm_mma(uint32_t d, const float* a_hi, const float* a_lo, const float* b_hi,
                                        const float* b_lo)
{
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int ao = s * 2 * (BtcSmem::kLboA / 4), bo = s * 64;  // two core matrices along K
        tc::mma_tf32(d, desc_kmajor_padded(a_hi + ao), tc::desc_kmajor(b_hi + bo), s > 0);
        tc::mma_tf32(d, desc_kmajor_padded(a_hi + ao), tc::desc_kmajor(b_lo + bo), 1);
        tc::mma_tf32(d, desc_kmajor_padded(a_lo + ao), tc::desc_kmajor(b_hi + bo), 1);
    }
}

constexpr int kBtcThreads = 512;

template <int P>
__global__ void __launch_bounds__(kBtcThreads, 1) k_blender_tc(Dev dv, const float* __restrict__ Btc, GasP g, BlendP bp, Ops ops,
                                                               int tr)
{
    static_assert(P == 4, "the tensor-core change of basis is the 64 x 64 matrix of degree 3");
    constexpr int N = 3, P3 = 64, R = tc::kRows;
    extern __shared__ __align__(128) float smem_btc[];
    __shared__ __align__(8) uint64_t bar_ld, bar_mma;
    __shared__ uint32_t tmem_base;
    __shared__ float s_part[4][6][tc::kRows];  // [mode group][sum][cell]
    float* sBhi = smem_btc + BtcSmem::oB;
    float* sBlo = sBhi + 64 * 64;
    float* sS = smem_btc + BtcSmem::oS;  // [5][R][64]
    float* sAhi = sS;                    // overlays the staging after the reads
    float* sAlo = sS + BtcSmem::kA;
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (dv.nc + tr - 1) / tr;  // tiles of tr <= R cells
    const float gm = f64_to_f32(g.gamma);
    if (warp == 0) tc::tmem_alloc(&tmem_base);
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
    bool ok = true, first = true, mma_out = false;  // mma_out: products issued, not yet waited for
    auto wait = [&](uint64_t* bar, uint32_t& ph) {
        bool done = false;
        for (int it = 0; it < (1 << 22) && !done; ++it) done = mbar_try_wait(bar, ph);
        ok = __syncthreads_and(done ? 1 : 0) != 0;
        if (ok) ph ^= 1;
    };
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t c0 = tile * tr;
        const int ncell = (int)((dv.nc - c0 < tr) ? dv.nc - c0 : tr);
        // ---- staging: one thread issues the copies (and, first, B)
        if (tid == 0) {
            const uint32_t bv = (uint32_t)(ncell * P3 * 4);
            mbar_arrive_expect_tx(&bar_ld, 5 * bv + (first ? (uint32_t)(BtcSmem::kB * 4) : 0u));
            if (first) tma_load_1d(sBhi, Btc, (uint32_t)(BtcSmem::kB * 4), &bar_ld);
#pragma unroll
            for (int v = 0; v < 5; ++v) tma_load_1d(sS + v * R * P3, dv.Uf + v * dv.nd + c0 * P3, bv, &bar_ld);
        }
        first = false;
        wait(&bar_ld, ph_ld);
        if (!ok) break;
        // ---- nodal values: thread t takes node t % 64 of cells 8 i + t / 64
        const int node = tid & 63;
        float x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int r = 8 * i + (tid >> 6);
            float val = 0.0f;
            if (r < ncell) {
                float cf[5];
#pragma unroll
                for (int v = 0; v < 5; ++v) cf[v] = sS[(v * R + r) * P3 + node];
                const int64_t dof = (c0 + r) * P3 + node;
                if (!positive_dof_screened(dv, dof, cf)) {
                    atomicMin(&s->bad_dof, (long long)dof);
                    s->err = PLENS_GPU_E_POSITIVITY;
                }
                const float p = get_p(cf, gm);
                val = (bp.var == 2) ? cf[0] : (bp.var == 1) ? p : p * cf[0];
            }
            x[i] = val;
        }
        __syncthreads();  // every staged value read: A may overlay the staging
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int r = 8 * i + (tid >> 6), o = a_off_padded(r, node);
            const float hi = tc::tf32_hi(x[i]);
            sAhi[o] = hi;
            sAlo[o] = x[i] - hi;
        }
        tc::fence_smem_async();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            cbm_mma(tmem, sAhi, sAlo, sBhi, sBlo);
            tc::mma_commit(&bar_mma);
        }
        mma_out = true;
        wait(&bar_mma, ph_mma);
        if (!ok) break;
        mma_out = false;
        tc::fence_after();
        // ---- partial sums: rows 32 (warp % 4) + lane, modes 16 (warp / 4) .. + 15
        {
            const int q = warp & 3, mg = warp >> 2, row = 32 * q + lane;
            float md[16];
            tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(16 * mg), md);
            float e0 = 0, e1 = 0, e2 = 0, asum = 0, ub = 0, tl = 0;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int n = 16 * mg + i, mi = n % P, mj = (n / P) % P, mk = n / (P * P);
                const float e = md[i] * md[i];
                e0 += e;
                if (mi < N && mj < N && mk < N) e1 += e;
                if (mi < N - 1 && mj < N - 1 && mk < N - 1) e2 += e;
                if (bp.do_filter) {
                    const float t = fabsf(md[i]);
                    asum += t;
                    const float xx = t * (ops.ftv[mi] + ops.ftv[mj] + ops.ftv[mk]);
                    ub += xx;
                    if (mi <= 1 && mj <= 1 && mk <= 1) tl += xx;
                }
            }
            s_part[mg][0][row] = e0;
            s_part[mg][1][row] = e1;
            s_part[mg][2][row] = e2;
            s_part[mg][3][row] = asum;
            s_part[mg][4][row] = ub;
            s_part[mg][5][row] = tl;
        }
        __syncthreads();
        // ---- this thread's cell (the first 128 threads): energies, TV-filter statistics, alpha
        const int64_t cell = c0 + tid;
        if (tid < ncell) {
            float e0 = 0, e1 = 0, e2 = 0, asum = 0, ub = 0, tl = 0;
#pragma unroll
            for (int mg = 0; mg < 4; ++mg) {
                e0 += s_part[mg][0][tid];
                e1 += s_part[mg][1][tid];
                e2 += s_part[mg][2][tid];
                asum += s_part[mg][3][tid];
                ub += s_part[mg][4][tid];
                tl += s_part[mg][5][tid];
            }
            float trouble = 1.0f - __fdividef(e1, e0);
            const float t2 = 1.0f - __fdividef(e2, e1);
            if (t2 > trouble) trouble = t2;
            const float thr = f64_to_f32(bp.thr), amin = f64_to_f32(bp.amin), amax = f64_to_f32(bp.amax);
            float alpha;
            if (bp.func == 0) {
                const float at = __fdividef(1.0f, 1.0f + __expf(-f64_to_f32(bp.sharp) * (__fdividef(trouble, thr) - 1.0f)));
                alpha = (at < amin) ? 0.0f : (at < amax ? at : amax);
            } else {
                const float at = __fdividef(trouble, thr);
                alpha = (at > 1.0f) ? 1.0f : at;
            }
            double ad = f32_to_f64(alpha);
            if (dv.cell_wall[cell]) {
                const double wl = eval_expr(dv, bp.expr_wall, 0, 0, 0, s->time);
                ad = (wl > ad) ? wl : ad;
            }
            dv.alpha_raw[cell] = ad;
            if (bp.do_filter) {
                dv.tvstat[cell] = f32_to_f64(asum);
                dv.tvstat[dv.nc + cell] = f32_to_f64(ub);
                dv.tvstat[2 * dv.nc + cell] = f32_to_f64(tl);
            }
        }
        tc::fence_before();
        __syncthreads();  // tensor memory read and shared memory free for the next tile
        tc::fence_after();
    }
    if (!ok) {
        if (tid == 0) s->err = PLENS_GPU_E_TIMEOUT;
        // copies or products still in flight land before the block leaves (bounded)
        for (int it = 0; it < (1 << 22) && !mbar_try_wait(&bar_ld, ph_ld); ++it) {
        }
        if (mma_out)
            for (int it = 0; it < (1 << 22) && !mbar_try_wait(&bar_mma, ph_mma); ++it) {
            }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem);
}

// The B operand of k_blender_tc on the host: C[mode][node] = C1[mi][ni] C1[mj][nj] C1[mk][nk]
// (mode = mi + 4 mj + 16 mk, node likewise) in FP64, rounded to FP32 and split into TF32 hi/lo,
// in the canonical K-major layout; then C's row sums (the modal coefficients of the constant 1),
// 2 x 64 x 64 + 64 floats in all.
inline void blender_tc_operand(const double* C1, float* out)
{
    constexpr int P = 4;
    for (int n = 0; n < 64; ++n) {
        double rs = 0;
        for (int k = 0; k < 64; ++k) {
            const int mi = n % P, mj = (n / P) % P, mk = n / (P * P);
            const int ni = k % P, nj = (k / P) % P, nk = k / (P * P);
            const float x = (float)(C1[mi * P + ni] * C1[mj * P + nj] * C1[mk * P + nk]);
            const float hi = tc::tf32_hi(x);
            out[tc::core_off(n, k)] = hi;
            out[64 * 64 + tc::core_off(n, k)] = x - hi;
            rs += x;
        }
        out[2 * 64 * 64 + n] = (float)rs;
    }
}

}  // namespace plens_gpu
