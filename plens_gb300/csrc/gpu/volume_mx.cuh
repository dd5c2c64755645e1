// volume_mx.cuh -- the mixed form's volume kernel for even P (N = 1, 3, 5) and the Chandrashekhar
// volume flux (the other volume fluxes take k_volume<P, float>): the same residual as
// k_volume (calc_cell_ho_inv_residual, calc_cell_ho_dif_residual, calc_cell_lo_inv_residual, the
// blend of calc_rhs and the register update; dgsem/plens.cc:3153-3583, 3753-3775, 4353-4400), with
// every per-block input staged in shared memory by TMA bulk copies. For even P each cell's P^3
// values of a variable are a multiple of 16 bytes, so a block's CPB cells are one contiguous,
// 16-byte aligned chunk per variable: one thread issues the copies, two mbarriers signal them --
// the FP32 state image (and, in the MIXED_R32 form, the FP32 metric images) that the flux phase
// needs first, then the FP64 state, the face values and the RK registers (and, in the MIXED form,
// 1/detJ in FP64), which arrive while the fluxes are computed. The first-order subcell residual
// of the troubled cells is the interior sums k_subcell_lo (subcell_mx.cuh) makes over the
// compacted troubled-cell list beside the face kernels, plus the cell-face terms, which this
// kernel adds from its staged face values.
//
// R64 selects the MIXED form: the residual's FP32 sums are scaled by -dt/detJ in FP64 (1/detJ
// made once from the FP64 det J), and the three FP64 RK registers are combined in FP64
// (update_rk4, dgsem/plens.cc:4353-4400). Its FP32 fluxes take the FP32 rounding of the FP64 Ja,
// read from the image made once at context creation: the values the threads would round from
// the FP64 array (f64_to_f32), bit for bit, with half the bytes and none of the nine conversions
// per node. Without R64 (MIXED_R32) the registers hold dt*R in FP32 and det J is read from its
// FP32 image as well.
#pragma once

#include <type_traits>

#include "async.cuh"
#include "kernels.cuh"

namespace plens_gpu {

// Shared-memory layout of one block (bytes), all regions 16-byte aligned.
template <int P, bool VISC, bool R64>
struct MxSmem {
    static constexpr int P2 = P * P, P3 = P2 * P, CPB = CellBlock<P>::CPB, NB = CPB * P3, NF = CPB * 6 * P2;
    static constexpr int NQ = 10;  // rho, 1/rho, v0, v1, v2, p, beta, ln rho, ln beta, |v|^2
    // per-cell strides of the node quantities and partial sums (16 banks between the cells at
    // P = 4) and of the FP32 metric terms; in the MIXED form the threads write the metric terms
    // (read from the FP32 image) in the swizzled order, the MIXED_R32 form stages the image as it
    // lies in memory
    static constexpr int PAD = (P == 4) ? 16 : 0;
    static constexpr int QCS = NQ * P3 + PAD, ACS = 15 * P3 + PAD;
    static constexpr bool JSW = R64 && P == 4;
    static constexpr int JCS = JSW ? P3 + PAD : P3, JMS = CPB * JCS;  // cell and component strides
    // the warps past the line tasks (phase A) and whether the MIXED form gives them the FP64
    // pre-update, which reads the two older registers from global memory (not staged)
    static constexpr int TPC = 3 * P2;
    static constexpr int TF = ((CPB * TPC + 31) / 32) * 32 < CellBlock<P>::THREADS ? ((CPB * TPC + 31) / 32) * 32
                                                                                    : CellBlock<P>::THREADS;
    static constexpr bool PRE = R64 && TF < CellBlock<P>::THREADS;
    static constexpr size_t RB = PRE ? 0 : (R64 ? 8 : 4);  // bytes of a staged register value
    static constexpr size_t up16(size_t x) { return (x + 15) / 16 * 16; }
    // staged inputs: the FP64 state (for the update), its FP32 image (for the fluxes), detJ (FP32
    // image; R64: 1/detJ in FP64), the FP32 metric terms (R64: rounded by the threads from FP64),
    // the RK registers, FP32 face values and auxiliary variables
    static constexpr size_t oU = 0;                                   // double [5][NB]
    static constexpr size_t oUf = oU + up16(8 * 5 * NB);              // float [5][NB]
    static constexpr size_t oDet = oUf + up16(4 * 5 * NB);            // float [NB] (R64: double [NB])
    static constexpr size_t oJ = oDet + up16((R64 ? 8 : 4) * NB);     // float [9][JMS]
    static constexpr size_t oR0 = oJ + up16(4 * 9 * JMS);             // RB [5][NB]
    static constexpr size_t oR1 = oR0 + up16(RB * 5 * NB);            // RB [5][NB]
    static constexpr size_t oSf = oR1 + up16(RB * 5 * NB);            // float [5][NF]
    static constexpr size_t oSf3 = oSf + up16(4 * 5 * NF);            // float [5][NF] (viscous)
    static constexpr size_t oAv = oSf3 + (VISC ? up16(4 * 5 * NF) : 0);  // float [9][NB] (viscous)
    static constexpr size_t oAcc = oAv + (VISC ? up16(4 * 9 * NB) : 0);  // float [CPB][ACS]: [15][P3]
    static constexpr size_t oQ = oAcc + up16(4 * CPB * ACS);          // float [CPB][QCS]: [NQ][P3]
    static constexpr size_t bytes = oQ + up16(4 * CPB * QCS);
};

// Resident blocks per SM the register allocation is sized for: 128-thread blocks at P = 2, 4 --
// six in the MIXED_R32 form (80 registers), seven in the MIXED form (72 registers, no spills;
// its 30 KB of shared memory allow seven) -- and two 224-thread blocks at P = 6.
template <int P, bool R64>
constexpr int vol_mx_min_blocks() { return P == 6 ? 2 : (R64 ? 7 : 6); }

template <int P, bool VISC, bool R64>
__global__ void __launch_bounds__(CellBlock<P>::THREADS, vol_mx_min_blocks<P, R64>()) k_volume_mx(Dev dv, Ops ops, GasP g, StageArgs sa)
{
    static_assert(P % 2 == 0, "bulk staging needs 16-byte aligned per-cell chunks (even P)");
    using CB = CellBlock<P>;
    using L = MxSmem<P, VISC, R64>;
    using RT = typename std::conditional<R64, double, float>::type;  // register storage type
    constexpr int P2 = CB::P2, P3 = CB::P3, CPB = CB::CPB, N = P - 1, NQ = L::NQ, NB = L::NB, NF = L::NF;
    constexpr int QCS = L::QCS, ACS = L::ACS, JCS = L::JCS, JMS = L::JMS;
    // index of node n in the metric-term array (swizzled where the threads write it)
    auto jx = [](int n) { return L::JSW ? swz<P>(n) : n; };
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2];
    double* stU = reinterpret_cast<double*>(smem_raw + L::oU);
    float* stUf = reinterpret_cast<float*>(smem_raw + L::oUf);
    float* stDet = reinterpret_cast<float*>(smem_raw + L::oDet);
    double* stInv = reinterpret_cast<double*>(smem_raw + L::oDet);  // R64: 1/detJ
    float* stJ = reinterpret_cast<float*>(smem_raw + L::oJ);
    RT* stR0 = reinterpret_cast<RT*>(smem_raw + L::oR0);
    RT* stR1 = reinterpret_cast<RT*>(smem_raw + L::oR1);
    float* stSf = reinterpret_cast<float*>(smem_raw + L::oSf);
    float* stSf3 = reinterpret_cast<float*>(smem_raw + L::oSf3);
    float* stAv = reinterpret_cast<float*>(smem_raw + L::oAv);
    float* sAcc = reinterpret_cast<float*>(smem_raw + L::oAcc);
    float* sQ = reinterpret_cast<float*>(smem_raw + L::oQ);

    Scalars* s = dv.sc;
    // no update after a positivity failure earlier in the step (the state stays that of the RHS
    // that failed, where the reference exits)
    if (!s->active || s->err) return;
    const int tid = threadIdx.x, cl = tid / P3, node = tid - cl * P3;
    const int64_t cell0 = (int64_t)blockIdx.x * CPB;
    const int ncb = (int)((dv.nc - cell0 < CPB) ? dv.nc - cell0 : CPB);  // cells of this block
    const int64_t cell = cell0 + cl;
    const bool valid = (cl < ncb);
    const bool need_r0 = sa.mode == 1 && sa.stage >= 3, need_r1 = sa.mode == 1 && sa.stage >= 2;

    // ---- staging: one thread issues the bulk copies
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const uint32_t bd = (uint32_t)(8 * ncb * P3), bf = (uint32_t)(4 * ncb * 6 * P2), bv = (uint32_t)(4 * ncb * P3);
        const uint32_t br = R64 ? bd : bv;  // one variable's chunk of a register
        const int64_t d0 = cell0 * P3, f0 = cell0 * 6 * P2;
        mbar_arrive_expect_tx(&bars[0], R64 ? bv * 5 : bv * (5 + 9 + 1));
#pragma unroll
        for (int v = 0; v < 5; ++v) tma_load_1d(stUf + v * NB, dv.Uf + v * dv.nd + d0, bv, &bars[0]);
        if (!R64) {
#pragma unroll
            for (int m = 0; m < 9; ++m) tma_load_1d(stJ + m * NB, dv.Jaf + m * dv.nd + d0, bv, &bars[0]);
            tma_load_1d(stDet, dv.detJf + d0, bv, &bars[0]);
        }
        // (with the FP64 pre-update the idle warp reads the registers itself)
        const bool st_r0 = need_r0 && !L::PRE, st_r1 = need_r1 && !L::PRE;
        uint32_t late = bd * 5 + bf * 5 + (st_r0 ? br * 5 : 0) + (st_r1 ? br * 5 : 0) + (VISC ? bf * 5 + bv * 9 : 0) +
                        (R64 ? bd : 0);
        mbar_arrive_expect_tx(&bars[1], late);
#pragma unroll
        for (int v = 0; v < 5; ++v) tma_load_1d(stU + v * NB, dv.U + v * dv.nd + d0, bd, &bars[1]);
#pragma unroll
        for (int v = 0; v < 5; ++v) tma_load_1d(stSf + v * NF, as_real<float>(dv.sf) + v * dv.nslot + f0, bf, &bars[1]);
        if (R64) tma_load_1d(stInv, dv.invJ + d0, bd, &bars[1]);
        if (st_r0)
#pragma unroll
            for (int v = 0; v < 5; ++v) tma_load_1d(stR0 + v * NB, as_real<RT>(sa.R0) + v * dv.nd + d0, br, &bars[1]);
        if (st_r1)
#pragma unroll
            for (int v = 0; v < 5; ++v) tma_load_1d(stR1 + v * NB, as_real<RT>(sa.R1) + v * dv.nd + d0, br, &bars[1]);
        if (VISC) {
#pragma unroll
            for (int v = 0; v < 5; ++v) tma_load_1d(stSf3 + v * NF, as_real<float>(dv.sf3) + v * dv.nslot + f0, bf, &bars[1]);
#pragma unroll
            for (int m = 0; m < 9; ++m) tma_load_1d(stAv + m * NB, as_real<float>(dv.avars) + m * dv.nd + d0, bv, &bars[1]);
        }
    }
    if (R64 && valid) {
        // the FP32 rounding of this node's metric terms, for the FP32 fluxes, from the image, into
        // the swizzled order (the loads are in flight while the first copy group lands; the
        // __syncthreads below publishes them)
        const int64_t dn = cell * P3 + node;
        float ja[9];
#pragma unroll
        for (int m = 0; m < 9; ++m) ja[m] = dv.Jaf[m * dv.nd + dn];
#pragma unroll
        for (int m = 0; m < 9; ++m) stJ[m * JMS + cl * JCS + jx(node)] = ja[m];
    }
    __syncthreads();  // barrier initialisation visible to every thread
    // the block takes one decision: a wait that ran out anywhere ends the block (error status set,
    // both copy groups waited for once more, bounded)
    if (!__syncthreads_and(mbar_wait0(&bars[0]) ? 1 : 0)) {
        if (tid == 0) s->err = PLENS_GPU_E_TIMEOUT;
        mbar_wait0(&bars[0]);
        mbar_wait0(&bars[1]);
        return;
    }

    const float gm = f64_to_f32(g.gamma);
    float* Q = sQ + cl * QCS;  // quantity k at node n of this cell: Q[k * P3 + swz(n)]
    const float* Cc = stUf + cl * P3;  // the FP32 state image: variable v at node n is Cc[v * NB + n]
    const float* J = stJ + cl * JCS;  // component m of Ja at node n of this cell: J[m * JMS + jx(n)]
    float* Acc = sAcc + cl * ACS;  // partial sum k at node n of this cell: Acc[k * P3 + swz(n)]
    const int sn = swz<P>(node), jn0 = jx(node);
    const int64_t dof = cell * P3 + node;
    const int bn = cl * P3 + node;  // node index within the block's staged chunks
    if (valid) {
        float c[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) c[v] = Cc[v * NB + node];
        const float p = get_p(c, gm);
        const float ri = 1.0f / c[0];
        const float v0 = c[1] * ri, v1 = c[2] * ri, v2 = c[3] * ri, beta = 0.5f * c[0] / p;
        Q[0 * P3 + sn] = c[0];
        Q[1 * P3 + sn] = ri;
        Q[2 * P3 + sn] = v0;
        Q[3 * P3 + sn] = v1;
        Q[4 * P3 + sn] = v2;
        Q[5 * P3 + sn] = p;
        Q[6 * P3 + sn] = beta;
        Q[7 * P3 + sn] = __logf(c[0]);
        Q[8 * P3 + sn] = __logf(beta);
        Q[9 * P3 + sn] = v0 * v0 + v1 * v1 + v2 * v2;
    }
    __syncthreads();
    const double alpha = valid ? dv.alpha[cell] : 0.0;
    const float alpha_t = f64_to_f32(alpha);

    bool late_waited = false, late_ok = true;
    // ---- phase A: two-point volume fluxes per line. The block's line tasks are numbered flat,
    // cell after cell, over the first TF threads (whole warps); the warps past them -- one at
    // P = 4 -- have no line task. In the MIXED form (an RK4 stage) those warps take the part of the
    // FP64 register update that does not depend on this stage's residual while the others compute
    // the fluxes: W = U + c1 R1 + c0 R0 and the node factor -dt/detJ, written over the staged U
    // and 1/detJ. GB300 issues FP64 at a small fraction of its FP32 rate; done here, that work
    // overlaps the FP32 flux phase instead of lengthening the update at the end.
    constexpr int TPC = L::TPC, TF = L::TF;  // line tasks per cell, threads running them
    const bool pre = L::PRE && sa.mode == 1;
    if (pre && tid >= TF) {
        // two nodes per pass, their register values loaded before the pass waits: the first
        // pass's loads overlap the wait for the late copy group (U and 1/detJ)
        const double* R0g = sa.R0 + cell0 * P3;
        const double* R1g = sa.R1 + cell0 * P3;
        const bool r0 = sa.stage >= 3, r1 = sa.stage >= 2;
        constexpr int NW = CB::THREADS - TF;  // threads of the spare warps
        for (int i = tid - TF; i < ncb * P3; i += 2 * NW) {
            const int j = i + NW;
            const bool two = j < ncb * P3;
            double a0[5], a1[5], b0[5], b1[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                a0[v] = r0 ? R0g[v * dv.nd + i] : 0.0;
                a1[v] = r1 ? R1g[v * dv.nd + i] : 0.0;
                b0[v] = (r0 && two) ? R0g[v * dv.nd + j] : 0.0;
                b1[v] = (r1 && two) ? R1g[v * dv.nd + j] : 0.0;
            }
            if (!late_waited) {
                late_ok = mbar_wait0(&bars[1]);
                late_waited = true;
            }
            if (!late_ok) break;
            stInv[i] = -stInv[i] * rhs_step(dv, cell0 + i / P3);
            if (two) stInv[j] = -stInv[j] * rhs_step(dv, cell0 + j / P3);
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                double w = stU[v * NB + i];
                if (r0) w = __fma_rn(sa.c0, a0[v], w);
                if (r1) w = __fma_rn(sa.c1, a1[v], w);
                stU[v * NB + i] = w;
                if (two) {
                    double x = stU[v * NB + j];
                    if (r0) x = __fma_rn(sa.c0, b0[v], x);
                    if (r1) x = __fma_rn(sa.c1, b1[v], x);
                    stU[v * NB + j] = x;
                }
            }
        }
        if (!late_waited) {
            late_ok = mbar_wait0(&bars[1]);
            late_waited = true;
        }
    }
    {
        const float hg = __fdividef(0.5f, gm - 1.0f), gf = __fdividef(gm, gm - 1.0f);
        for (int ft = tid; ft < CPB * TPC && tid < TF; ft += TF) {
            // P = 4: warp dir, lanes (cell, line); otherwise the tasks of a cell in a row
            int tc, dir, line;
            if constexpr (P == 4 && CPB == 2 && TF == 96) {
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
            const float* Qa = sQ + tc * QCS;
            const float* Ca = stUf + tc * P3;
            const float* Jt = stJ + tc * JCS;
            float* At = sAcc + tc * ACS;
            const int la = line % P, lb = line / P;
            float acc[P][5];
#pragma unroll
            for (int i = 0; i < P; ++i)
#pragma unroll
                for (int v = 0; v < 5; ++v) acc[i][v] = 0.0f;
            // Chandrashekhar (the only volume flux this kernel is launched for): unnormalised
            // directions, per-node logarithms; the diagonal term only at the two end nodes
            // (D_ii = 0 at interior GLL nodes)
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int ni = line_node<P>(dir, la, lb, i), qni = swz<P>(ni), jni = jx(ni);
                float qi[10];
#pragma unroll
                for (int k = 0; k < 10; ++k) qi[k] = Qa[k * P3 + qni];
                const float ji[3] = {Jt[(dir * 3) * JMS + jni], Jt[(dir * 3 + 1) * JMS + jni], Jt[(dir * 3 + 2) * JMS + jni]};
                if (i == 0 || i == N) {
                    float F[5];
                    chandrashekhar_same_f32(qi, ji, gf, F);
                    const float dd = opD2<float>(ops, i * P + i);
#pragma unroll
                    for (int v = 0; v < 5; ++v) acc[i][v] += dd * F[v];
                }
#pragma unroll
                for (int m = i + 1; m < P; ++m) {
                    const int nm = line_node<P>(dir, la, lb, m), qnm = swz<P>(nm), jnm = jx(nm);
                    float qm[10];
#pragma unroll
                    for (int k = 0; k < 10; ++k) qm[k] = Qa[k * P3 + qnm];
                    const float nv[3] = {ji[0] + Jt[(dir * 3) * JMS + jnm], ji[1] + Jt[(dir * 3 + 1) * JMS + jnm],
                                         ji[2] + Jt[(dir * 3 + 2) * JMS + jnm]};
                    float F[5];
                    chandrashekhar_pair_f32(qi, qm, nv, hg, F);
                    const float di = opD<float>(ops, i * P + m), dm = opD<float>(ops, m * P + i);
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        acc[i][v] += di * F[v];
                        acc[m][v] += dm * F[v];
                    }
                }
            }
            // surface term of the line's two end nodes, which lie on faces 2 dir and 2 dir + 1 at
            // face dof la + P lb (calc_cell_ho_inv_residual, dgsem/plens.cc:3237-3268):
            // -sign (F* - F_in(n/|n|)) |n| / w = -sign (F* |n| - F_in(n)) / w, the physical flux
            // being linear in n. Every lane of a warp takes both ends; per node the surface terms
            // would diverge (a corner node has three, an interior node none). Needs the face
            // values of the late copy group: each thread waits for it once (bounded; the block
            // decides on the outcome below).
            if (!late_waited) {
                late_ok = mbar_wait0(&bars[1]);
                late_waited = true;
            }
            if (late_ok) {
                const float* sfa = stSf + tc * 6 * P2;
                const int q = la + P * lb;
#pragma unroll
                for (int lr = 0; lr < 2; ++lr) {
                    const int i = lr ? N : 0;
                    const int ni = line_node<P>(dir, la, lb, i);
                    const int f = 2 * dir + lr;
                    const int jni = jx(ni);
                    const float jn[3] = {Jt[(dir * 3) * JMS + jni], Jt[(dir * 3 + 1) * JMS + jni], Jt[(dir * 3 + 2) * JMS + jni]};
                    const float nn = sqrtf(jn[0] * jn[0] + jn[1] * jn[1] + jn[2] * jn[2]);
                    const float ci[5] = {Ca[ni], Ca[NB + ni], Ca[2 * NB + ni], Ca[3 * NB + ni], Ca[4 * NB + ni]};
                    float fin[5];
                    inv_flux(ci, jn, gm, fin);
                    const float ss = lr ? -1.0f : 1.0f;
                    const float rw = __fdividef(1.0f, opW<float>(ops, lr * N));
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        const float fs = -ss * sfa[v * NF + f * P2 + q];
                        acc[i][v] += -ss * (fs * nn - fin[v]) * rw;
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int qni = swz<P>(line_node<P>(dir, la, lb, i));
#pragma unroll
                for (int v = 0; v < 5; ++v) At[(dir * 5 + v) * P3 + qni] = acc[i][v];
            }
        }
    }
    // face values, registers (and viscous inputs) staged; partial sums visible
    if (!__syncthreads_and((late_ok && mbar_wait0(&bars[1])) ? 1 : 0)) {
        if (tid == 0) s->err = PLENS_GPU_E_TIMEOUT;
        mbar_wait0(&bars[1]);
        return;
    }

    // ---- phase B: HO inviscid = volume + surface (summed per direction in phase A), scaled by
    // 1/(-detJ)
    const int ti[3] = {node % P, (node / P) % P, node / P2};
    // R64: the parts of the residual stay unscaled FP32 sums, scaled by -dt/detJ in FP64 in phase D
    const float detJ = (valid && !R64) ? stDet[bn] : 1.0f;
    float ho[5] = {0, 0, 0, 0, 0};
    if (valid) {
        const float js = R64 ? 1.0f : __fdividef(-1.0f, detJ);
#pragma unroll
        for (int v = 0; v < 5; ++v) ho[v] = (Acc[v * P3 + sn] + Acc[(5 + v) * P3 + sn] + Acc[(10 + v) * P3 + sn]) * js;
    }

    // ---- viscous HO residual: nodal viscous fluxes along each contravariant direction
    float hd[5] = {0, 0, 0, 0, 0};
    if (VISC) {
        __syncthreads();  // Acc is reused
        float av[9];
#pragma unroll
        for (int m = 0; m < 9; ++m) av[m] = valid ? stAv[m * NB + bn] : 0.0f;
        if (valid) {
            const float ci[5] = {Cc[node], Cc[NB + node], Cc[2 * NB + node], Cc[3 * NB + node], Cc[4 * NB + node]};
#pragma unroll
            for (int md = 0; md < 3; ++md) {
                const float jn[3] = {J[(md * 3) * JMS + jn0], J[(md * 3 + 1) * JMS + jn0], J[(md * 3 + 2) * JMS + jn0]};
                float F[5];
                dif_flux(ci, av, jn, F);  // linear in the direction: F(n/|n|) |n| = F(n)
#pragma unroll
                for (int v = 0; v < 5; ++v) Acc[(md * 5 + v) * P3 + sn] = F[v];
            }
        }
        __syncthreads();
        if (valid) {
            for (int m = 0; m < P; ++m) {
#pragma unroll
                for (int md = 0; md < 3; ++md) {
                    const int lo = (md == 0) ? m + P * ti[1] + P2 * ti[2] : (md == 1) ? ti[0] + P * m + P2 * ti[2] : ti[0] + P * ti[1] + P2 * m;
                    const float dvl = opD<float>(ops, ti[md] * P + m);
#pragma unroll
                    for (int v = 0; v < 5; ++v) hd[v] += dvl * Acc[(md * 5 + v) * P3 + swz<P>(lo)];
                }
            }
            const float ci[5] = {Cc[node], Cc[NB + node], Cc[2 * NB + node], Cc[3 * NB + node], Cc[4 * NB + node]};
            const float* sf3b = stSf3 + cl * 6 * P2;
#pragma unroll
            for (int sd = 0; sd < 3; ++sd) {
#pragma unroll
                for (int lr = 0; lr < 2; ++lr) {
                    if (ti[sd] != (lr ? N : 0)) continue;
                    const int f = 2 * sd + lr;
                    const int q = (sd == 0) ? ti[1] + P * ti[2] : (sd == 1) ? ti[0] + P * ti[2] : ti[0] + P * ti[1];
                    const float jn[3] = {J[(sd * 3) * JMS + jn0], J[(sd * 3 + 1) * JMS + jn0], J[(sd * 3 + 2) * JMS + jn0]};
                    const float nn = sqrtf(jn[0] * jn[0] + jn[1] * jn[1] + jn[2] * jn[2]);
                    float fin[5];
                    dif_flux(ci, av, jn, fin);
                    const float ss = lr ? -1.0f : 1.0f;
                    const float rw = __fdividef(1.0f, opW<float>(ops, lr * N));
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        const float fs = -ss * sf3b[v * NF + f * P2 + q];
                        hd[v] += -ss * (fs * nn - fin[v]) * rw;
                    }
                }
            }
            if (!R64) {
                const float js = __fdividef(1.0f, detJ);
#pragma unroll
                for (int v = 0; v < 5; ++v) hd[v] *= js;
            }
        }
    }

    // ---- phase C: first-order subcell residual, only where alpha > 0: the interior sums
    // k_subcell_lo wrote at this cell's dofs (it takes every cell of the list, the cells whose
    // stored alpha passes this same test), plus the cell-face terms at the nodes on the cell's
    // faces: this stage's face flux x |Ja| / w (contribution sign x flux sign = +1,
    // calc_cell_lo_inv_residual, dgsem/plens.cc:3544-3575)
    float lo[5] = {0, 0, 0, 0, 0};
    if (valid && stored_gt0<float>(alpha)) {
        {
#pragma unroll
            for (int v = 0; v < 5; ++v) lo[v] = dv.lo_buf[v * dv.nd + dof];
            const float* sfa = stSf + cl * 6 * P2;
#pragma unroll
            for (int sd = 0; sd < 3; ++sd) {
#pragma unroll
                for (int lr = 0; lr < 2; ++lr) {
                    if (ti[sd] != (lr ? N : 0)) continue;
                    const int f = 2 * sd + lr;
                    const int q = (sd == 0) ? ti[1] + P * ti[2] : (sd == 1) ? ti[0] + P * ti[2] : ti[0] + P * ti[1];
                    const float j0 = J[(sd * 3) * JMS + jn0], j1 = J[(sd * 3 + 1) * JMS + jn0], j2 = J[(sd * 3 + 2) * JMS + jn0];
                    const float sw = __fdividef(sqrtf(j0 * j0 + j1 * j1 + j2 * j2), opW<float>(ops, lr * N));
#pragma unroll
                    for (int v = 0; v < 5; ++v) lo[v] += sfa[v * NF + f * P2 + q] * sw;
                }
            }
            const float js = R64 ? 1.0f : __fdividef(-1.0f, detJ);
#pragma unroll
            for (int v = 0; v < 5; ++v) lo[v] *= js;
        }
    }
    if (!valid) return;

    if constexpr (R64) {
        // ---- phase D (MIXED): blend of the unscaled FP32 sums,
        // R = (-1/detJ) (alpha lo + (1 - alpha) ho - (1 - alpha_d) hd), scaled in FP64; dt*R, the
        // three registers and their combination in FP64
        const float ad = VISC ? f64_to_f32(dv.alpha_d[cell]) : 0.0f;
        double Ru[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            float r = alpha_t * lo[v] + (1.0f - alpha_t) * ho[v];
            if (VISC) r -= (1.0f - ad) * hd[v];
            Ru[v] = f32_to_f64(r);
        }
        if (g.plens_2d) Ru[3] = 0.0;
        if (sa.mode == 0) {
            const double nij = -stInv[bn];
#pragma unroll
            for (int v = 0; v < 5; ++v) sa.Rout[v * dv.nd + dof] = Ru[v] * nij;
            return;
        }
        // -dt/detJ: made by the idle warp during phase A when it exists
        const double sc = pre ? stInv[bn] : -stInv[bn] * rhs_step(dv, cell);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const double Rs = Ru[v] * sc;
            const int64_t k = v * dv.nd + dof;
            const double u = stU[v * NB + bn];
            double un;
            if (sa.mode == 1) {
                // U + c0 R0 + c1 R1 + c2 Rs as a chain of FP64 multiply-adds (one rounding each);
                // with the idle warp, stU already holds W = U + c0 R0 + c1 R1
                if (pre) {
                    un = __fma_rn(sa.c2, Rs, u);
                } else {
                    un = u;
                    if (sa.stage >= 3) un = __fma_rn(sa.c0, stR0[v * NB + bn], un);
                    if (sa.stage >= 2) un = __fma_rn(sa.c1, stR1[v * NB + bn], un);
                    un = __fma_rn(sa.c2, Rs, un);
                }
                if (sa.keep) sa.Rw[k] = Rs;
            } else {
                if (sa.stage == 1) un = u + Rs;
                else if (sa.stage == 2) un = 0.75 * dv.U0[k] + 0.25 * u + 0.25 * Rs;
                else un = 1.0 / 3 * dv.U0[k] + 2.0 / 3 * u + 2.0 / 3 * Rs;
            }
            dv.U[k] = un;
            dv.Uf[k] = f64_to_f32(un);
        }
        return;
    }

    // ---- phase D (MIXED_R32): blend and register combination in FP32 (the residual is an FP32
    // result, and so is dt*R, which the registers hold in FP32); the state accumulated in FP64
    float R[5];
    const float ad = VISC ? f64_to_f32(dv.alpha_d[cell]) : 0.0f;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        if (VISC) R[v] = (1.0f - ad) * hd[v] + alpha_t * lo[v] + (1.0f - alpha_t) * ho[v];
        else R[v] = alpha_t * lo[v] + (1.0f - alpha_t) * ho[v];
    }
    if (g.plens_2d) R[3] = 0.0f;
    if (sa.mode == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) sa.Rout[v * dv.nd + dof] = f32_to_f64(R[v]);
        return;
    }
    const float dtu = f64_to_f32(rhs_step(dv, cell));
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        const float Rs = R[v] * dtu;
        const int64_t k = v * dv.nd + dof;
        const double u = stU[v * NB + bn];
        if (sa.mode == 1) {
            float inc;
            if (sa.stage == 1) inc = sa.fc2 * Rs;
            else if (sa.stage == 2) inc = sa.fc1 * (float)stR1[v * NB + bn] + sa.fc2 * Rs;
            else inc = sa.fc0 * (float)stR0[v * NB + bn] + sa.fc1 * (float)stR1[v * NB + bn] + sa.fc2 * Rs;
            if (sa.keep) as_real<float>(sa.Rw)[k] = Rs;
            const double un = u + f32_to_f64(inc);
            dv.U[k] = un;
            dv.Uf[k] = f64_to_f32(un);
        } else {
            const double Rsd = f32_to_f64(Rs);
            double un;
            if (sa.stage == 1) un = u + Rsd;
            else if (sa.stage == 2) un = 0.75 * dv.U0[k] + 0.25 * u + 0.25 * Rsd;
            else un = 1.0 / 3 * dv.U0[k] + 2.0 / 3 * u + 2.0 / 3 * Rsd;
            dv.U[k] = un;
            dv.Uf[k] = f64_to_f32(un);
        }
    }
}

}  // namespace plens_gpu
