// subcell_mx.cuh -- the mixed forms' first-order subcell residual over the compacted troubled-cell
// list: calc_cell_lo_inv_residual (dgsem/plens.cc:3469-3583) for the cells with alpha > 0 only,
// in a kernel of its own on the indicator stream, beside the face kernels.
//
// The list is ordered by cell index and built without atomics, the same on every run. The
// smoothing kernel (k_alpha_smooth, 128 cells per block) writes each block's troubled-cell count
// and its four warp ballots. k_subcell_lo then finds the cell at each list position itself: every
// block takes the prefix sums of the counts into shared memory, and a position maps to its
// smoothing block by a binary search there and to its cell by the rank among the block's ballot
// bits. (Meshes whose counts do not fit there take k_lo_list first, which writes the list from
// the same counts and ballots.) It runs the subcell interfaces inside each listed cell (the line
// tasks' P - 1 interior fluxes) and writes the cell's unscaled sums of the three directions to
// lo_buf[var][cell dofs]. It needs the state, the metric terms and alpha only; the cell-face terms
// of the first-order residual (the inviscid face flux x |Ja| / w at the nodes on the cell's faces,
// plens.cc:3544-3575) need this stage's face fluxes and are added by the volume kernel, which has
// them staged.
#pragma once

#include "kernels.cuh"

namespace plens_gpu {

// the most smoothing-block prefix sums (ints, 32 KB) the subcell kernel takes into shared memory
constexpr int kLoDecodeMaxBlocks = 8192;

// The troubled cells in cell order, lo_list[pos] = cell, and *lo_count, from the smoothing
// kernel's block counts and ballots (meshes whose counts do not fit k_subcell_lo's shared memory)
static __global__ void __launch_bounds__(kSmoothThreads) k_lo_list(Dev dv)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    __shared__ int s_part[kSmoothThreads / 32];
    __shared__ int s_off;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int b = blockIdx.x;
    // offset of this block: the troubled cells of the blocks before it
    int part = 0;
    for (int j = tid; j < b; j += kSmoothThreads) part += dv.lo_blk[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) s_part[warp] = part;
    __syncthreads();
    if (tid == 0) {
        int t = 0;
        for (int w = 0; w < kSmoothThreads / 32; ++w) t += s_part[w];
        s_off = t;
    }
    __syncthreads();
    const int64_t c = (int64_t)b * kSmoothThreads + tid;
    const unsigned m = dv.lo_mask[4 * b + warp];
    const bool flag = (m >> lane) & 1u;
    int wofs = 0;
    for (int w = 0; w < warp; ++w) wofs += __popc(dv.lo_mask[4 * b + w]);
    const int pos = s_off + wofs + __popc(m & ((1u << lane) - 1u));
    if (flag && c < dv.nc) dv.lo_list[pos] = (int32_t)c;
    if (b == (int)gridDim.x - 1 && tid == 0) *dv.lo_count = s_off + dv.lo_blk[b];
}

// list position p -> cell, from the exclusive prefix sums pre[0..nblk] of the smoothing blocks'
// troubled-cell counts (pre[nblk] = the list's length) and their ballots: the block is the last
// one whose prefix does not exceed p, the cell the (p - prefix)-th set bit of its ballots
__device__ __forceinline__ int32_t lo_decode(int p, const int* pre, int nblk, const uint32_t* mask)
{
    int lo = 0, hi = nblk;  // pre[lo] <= p < pre[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pre[mid] <= p) lo = mid;
        else hi = mid;
    }
    int r = p - pre[lo];
    const uint4 m4 = reinterpret_cast<const uint4*>(mask)[lo];
    const unsigned w[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int cnt = __popc(w[k]);
        if (r < cnt) {
            unsigned x = w[k];
            for (int i = 0; i < r; ++i) x &= x - 1u;  // clear the r lowest set bits
            return (int32_t)(lo * kSmoothThreads + 32 * k + (__ffs(x) - 1));
        }
        r -= cnt;
    }
    return -1;
}

// Interior subcell sums of the listed cells, CPB cells per block, one thread per GLL node; line
// tasks numbered flat over the block's cells (3 P^2 per cell), each running the P - 1 subcell
// interfaces of one line. The grid is persistent: blocks take groups of CPB listed cells with a
// stride, up to the count the list kernel wrote, and the loads are pipelined: while a group's
// fluxes run, every thread has its node's state image and metric terms of the block's next group
// in flight in registers, and the threads of the first CPB lanes the list entries of the group
// after it. A group then waits for no global load; only the block's first group does. HLLC --
// whose subcell flux does not read alpha -- has an instantiation of its own without the alpha
// load or the scheme switch. The metric terms are read from the FP32 image both mixed forms
// keep. The launcher caps the grid at four blocks per SM.
template <int P, bool HLLC>
__global__ void __launch_bounds__(CellBlock<P>::THREADS) k_subcell_lo(Dev dv, Ops ops, GasP g)
{
    using CB = CellBlock<P>;
    constexpr int P2 = CB::P2, P3 = CB::P3, CPB = CB::CPB;
    constexpr int TPC = 3 * P2;
    // node arrays in the swizzled order with the cells 16 banks apart at P = 4 (swz, device.cuh)
    constexpr int PAD = (P == 4) ? 16 : 0, CS = P3 + PAD, NBS = CPB * CS, ACS = 15 * P3 + PAD;
    __shared__ float sC[5][NBS];  // FP32 state image: variable v of node n of cell c at [v][c CS + swz(n)]
    __shared__ float sJ[9][NBS];  // FP32 rounding of Ja, the same order
    __shared__ float sAcc[CPB * ACS];  // partial sum k of node n of cell c at [c ACS + k P3 + swz(n)]
    __shared__ float sAl[CPB];
    __shared__ int32_t sCell[2][CPB];  // cells of this group and of the block's next group
    __shared__ int sW[CB::THREADS / 32];
    extern __shared__ int sPre[];  // decoding: [nblk + 1] prefix sums of the block counts
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int tid = threadIdx.x, cl = tid / P3, node = tid - cl * P3, lane = tid & 31, warp = tid >> 5;
    const float gm = f64_to_f32(g.gamma);
    const int G = gridDim.x;
    const float* Ja = dv.Jaf;
    const bool decode = dv.lo_decode != 0;
    const int nblk = (int)((dv.nc + kSmoothThreads - 1) / kSmoothThreads);
    int n = 0;  // the list's length
    if (decode) {
        // the exclusive prefix sums of the smoothing blocks' counts: each thread scans a chunk,
        // the chunk sums are scanned across the block, the chunks are rewritten with offsets
        for (int i = tid; i < nblk; i += CB::THREADS) sPre[i] = dv.lo_blk[i];
        __syncthreads();
        const int chunk = (nblk + CB::THREADS - 1) / CB::THREADS;
        const int b0 = tid * chunk, b1 = (b0 + chunk < nblk) ? b0 + chunk : nblk;
        int sum = 0;
        for (int i = b0; i < b1; ++i) sum += sPre[i];
        int x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sW[warp] = x;
        __syncthreads();
        int run = x - sum, total = 0;
        for (int w = 0; w < CB::THREADS / 32; ++w) {
            if (w < warp) run += sW[w];
            total += sW[w];
        }
        for (int i = b0; i < b1; ++i) {
            const int v = sPre[i];
            sPre[i] = run;
            run += v;
        }
        if (tid == 0) sPre[nblk] = total;
        __syncthreads();
        n = total;
        if (blockIdx.x == 0 && tid == 0) *dv.lo_count = n;
    } else if (tid < CPB) {
        n = *dv.lo_count;
    }
    // the cell at list position p (-1 past the end); decoding also writes the list entry
    auto entry = [&](int p) -> int32_t {
        if (decode) {
            if (p >= n) return -1;
            const int32_t c = lo_decode(p, sPre, nblk, dv.lo_mask);
            dv.lo_list[p] = c;
            return c;
        }
        const int32_t c = (p < dv.nc) ? dv.lo_list[p] : -1;
        return (p < n) ? c : -1;
    };
    // the first two groups' cells
    if (tid < CPB) {
#pragma unroll
        for (int j = 0; j < 2; ++j) sCell[j][tid] = entry((blockIdx.x + j * G) * CPB + tid);
    }
    __syncthreads();
    if (sCell[0][0] < 0) return;  // the list ends before this block's first group
    // this thread's node of the first group
    float pc[5] = {0, 0, 0, 0, 0}, pa = 0.0f, pj[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    auto fetch = [&](int32_t c) {
        if (c < 0) return;
        const int64_t dof = (int64_t)c * P3 + node;
#pragma unroll
        for (int v = 0; v < 5; ++v) pc[v] = dv.Uf[v * dv.nd + dof];
#pragma unroll
        for (int m = 0; m < 9; ++m) pj[m] = Ja[m * dv.nd + dof];
    };
    if (cl < CPB) fetch(sCell[0][cl]);
    if (!HLLC && tid < CPB && sCell[0][tid] >= 0) pa = f64_to_f32(dv.alpha[sCell[0][tid]]);
    for (int k = 0;; ++k) {
        const int cur = k & 1;
        const int ncb = (CPB == 1 || sCell[cur][CPB - 1] >= 0) ? CPB : [&] {
            int q = 1;
            while (q < CPB && sCell[cur][q] >= 0) ++q;
            return q;
        }();
        const int32_t mycell = (cl < ncb) ? sCell[cur][cl] : -1;  // this thread's cell of the group
        // this group's node values, fetched during the previous group
        if (cl < ncb) {
            const int bn = cl * CS + swz<P>(node);
#pragma unroll
            for (int v = 0; v < 5; ++v) sC[v][bn] = pc[v];
#pragma unroll
            for (int m = 0; m < 9; ++m) sJ[m][bn] = pj[m];
        }
        if (!HLLC && tid < CPB) sAl[tid] = pa;
        __syncthreads();
        // in flight during the fluxes: the next group's node values, the list entries after it
        int32_t after = -1;
        if (cl < CPB) fetch(sCell[cur ^ 1][cl]);
        if (tid < CPB) {
            after = entry((blockIdx.x + (k + 2) * G) * CPB + tid);
            if (!HLLC && sCell[cur ^ 1][tid] >= 0) pa = f64_to_f32(dv.alpha[sCell[cur ^ 1][tid]]);
        }
        for (int ft = tid; ft < CPB * TPC; ft += CB::THREADS) {
            // P = 4: warp dir, lanes (cell, line); otherwise the tasks of a cell in a row
            int tc, dir, line;
            if constexpr (P == 4 && CPB == 2) {
                dir = ft >> 5;
                tc = (ft >> 4) & 1;
                line = ft & 15;
            } else {
                tc = ft / TPC;
                const int task = ft - tc * TPC;
                dir = task / P2;
                line = task - dir * P2;
            }
            if (tc >= ncb) continue;
            float fb = 0.0f;
            if (!HLLC) {
                const float at = sAl[tc];
                fb = (at <= 0.0f) ? 0.0f : (at <= 1.0f ? at : 1.0f);  // the cell's alpha as flux blender (plens.cc:3492)
            }
            const int la = line % P, lb = line / P;
            const int base = tc * CS;
            float acc[P][5];
#pragma unroll
            for (int i = 0; i < P; ++i)
#pragma unroll
                for (int v = 0; v < 5; ++v) acc[i][v] = 0.0f;
            // running subcell normal n_(i-1,i) = Ja_0 + sum_{l<i} sum_m Q_lm Ja_m (metric_terms.cc:106-141)
            const int n0 = base + swz<P>(line_node<P>(dir, la, lb, 0));
            float sn[3] = {sJ[dir * 3][n0], sJ[dir * 3 + 1][n0], sJ[dir * 3 + 2][n0]};
#pragma unroll
            for (int id = 1; id < P; ++id) {
#pragma unroll
                for (int m = 0; m < P; ++m) {
                    const int nm = base + swz<P>(line_node<P>(dir, la, lb, m));
                    const float qlm = opQ<float>(ops, (id - 1) * P + m);
#pragma unroll
                    for (int d = 0; d < 3; ++d) sn[d] += qlm * sJ[dir * 3 + d][nm];
                }
                const int nl = base + swz<P>(line_node<P>(dir, la, lb, id - 1)), nr = base + swz<P>(line_node<P>(dir, la, lb, id));
                const float nn = sqrtf(sn[0] * sn[0] + sn[1] * sn[1] + sn[2] * sn[2]);
                const float dn[3] = {__fdividef(sn[0], nn), __fdividef(sn[1], nn), __fdividef(sn[2], nn)};
                const float cL[5] = {sC[0][nl], sC[1][nl], sC[2][nl], sC[3][nl], sC[4][nl]};
                const float cR[5] = {sC[0][nr], sC[1][nr], sC[2][nr], sC[3][nr], sC[4][nr]};
                float F[5];
                if (HLLC) hllc_n_f32(cL, cR, dn, gm, F);
                else inv_surf_flux_mx(cL, cR, dn, gm, g.isf, fb, F);
                const float wl = __fdividef(nn, opW<float>(ops, id - 1)), wr = __fdividef(nn, opW<float>(ops, id));
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    acc[id - 1][v] += F[v] * wl;
                    acc[id][v] -= F[v] * wr;
                }
            }
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int ni = tc * ACS + swz<P>(line_node<P>(dir, la, lb, i));
#pragma unroll
                for (int v = 0; v < 5; ++v) sAcc[ni + (dir * 5 + v) * P3] = acc[i][v];
            }
        }
        __syncthreads();
        if (cl < ncb) {
            const int64_t o = (int64_t)mycell * P3 + node;  // the cell's own dofs
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                const int a = cl * ACS + v * P3 + swz<P>(node);
                dv.lo_buf[v * dv.nd + o] = sAcc[a] + sAcc[a + 5 * P3] + sAcc[a + 10 * P3];
            }
        }
        // the group after next takes this group's slot; the shared arrays are reused
        if (tid < CPB) sCell[cur][tid] = after;
        __syncthreads();
        if (sCell[cur ^ 1][0] < 0) break;  // the block's next group is empty (the same for the whole block)
    }
}

}  // namespace plens_gpu
