// kernels.cuh -- the hot-path kernels, templated on P = N+1 and on the arithmetic type T
// (double: plain path; float: the mixed forms, whose state is FP64 and whose RK registers, metric
// terms and register accumulation are FP64 in the MIXED form and FP32 in the MIXED_R32 form, see
// plens_precision). One block handles CellBlock<P>::CPB cells with one thread per GLL node.
#pragma once

#include "device.cuh"
#include "flux.cuh"

namespace plens_gpu {

struct StageArgs {
    int mode;        // 0: write the unscaled residual to Rout; 1: RK4 stage; 2: RK3 stage
    int stage;       // 1..5 (RK4) or 1..3 (RK3)
    double* Rout;
    double* Rw;      // register receiving dt*R (RK4)
    const double* R0;
    const double* R1;
    double c0, c1, c2;
    float fc0, fc1, fc2;  // the same coefficients for the MIXED_R32 form's FP32 register combination
    int reg64;  // mixed forms: 1 (MIXED) FP64 registers, FP64 1/detJ scaling and accumulation; 0 (MIXED_R32) FP32
    int keep;   // RK4: 1 when a later stage reads this stage's register (every stage but the last)
};

// ------------------------------------------------------------------------ step bookkeeping

static __global__ void k_step_begin(Dev dv, double end_time)
{
    Scalars* s = dv.sc;
    s->end_time = end_time;
    s->active = (s->err == 0 && s->time < end_time) ? 1 : 0;
    s->dtmin = ord_double(1e6);
}

// dt after the global min-reduction; the clip to end_time affects the clock only, the RHS is
// multiplied by the unclipped value (loc_time_steps is set before the clip in update_rk4,
// dgsem/plens.cc:3903-3911 and 4339-4341)
static __global__ void k_dt_finalize(Dev dv)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    const double dt = unord_double(s->dtmin);
    s->dt_update = dt;
    s->dt = (dt > (s->end_time - s->time)) ? s->end_time - s->time : dt;
}

// FP32 rounding of an FP64 array (the mixed form's metric images)
static __global__ void k_round_f32(const double* __restrict__ in, float* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = f64_to_f32(in[i]);
}

// FP64 reciprocal of an FP64 array (the MIXED form's 1/detJ)
static __global__ void k_reciprocal(const double* __restrict__ in, double* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = 1.0 / in[i];
}

// The state from (and to) a page-locked host buffer read through its device mapping: one pass
// over the host link that also writes the mixed form's FP32 image.
static __global__ void k_state_in(Dev dv, const double* __restrict__ src)
{
    const int64_t n = 5 * dv.nd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double u = src[i];
        dv.U[i] = u;
        if (dv.Uf) dv.Uf[i] = f64_to_f32(u);
    }
}

static __global__ void k_state_out(Dev dv, double* __restrict__ dst)
{
    const int64_t n = 5 * dv.nd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = dv.U[i];
}

// the device scalars into a page-locked, device-mapped host mirror, read by the host once the
// stream has synchronised: no copy engine is involved, so the read never waits behind bulk
// host <-> device copies in flight on other streams
static __global__ void k_scalars_out(Dev dv, Scalars* __restrict__ dst)
{
    *dst = *dv.sc;
    __threadfence_system();
}

// the outcome of one member of a sequence of states (plens_gpu_advance_states)
struct MemberStatus {
    double time;
    long long n_steps, bad_dof;
    int err, pad;
};

// a member's outcome into a page-locked, device-mapped host array (no copy engine involved)
static __global__ void k_member_status(Dev dv, MemberStatus* __restrict__ dst)
{
    const Scalars* s = dv.sc;
    dst->time = s->time;
    dst->n_steps = s->n_steps;
    dst->bad_dof = s->bad_dof;
    dst->err = s->err;
    __threadfence_system();
}

// the clock of the next state of a sequence (plens_gpu_advance_states), on the stream: what
// plens_gpu_set_time writes from the host
static __global__ void k_set_clock(Dev dv, double t, long long n_steps)
{
    Scalars* s = dv.sc;
    s->time = t;
    s->n_steps = n_steps;
    s->err = 0;
    s->bad_dof = INT64_MAX;
}

// mixed form: the FP32 image of the state after the host or a restore changed U
static __global__ void k_state_image(Dev dv)
{
    const int64_t n = 5 * dv.nd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dv.Uf[i] = f64_to_f32(dv.U[i]);
}

// step-start snapshot of the state and the clock (learned sensor): U0 = U
static __global__ void k_snapshot(Dev dv)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int64_t n2 = 5 * dv.nd / 2;  // nd = cells * P^3; 5 * nd may be odd
    const double2* src = reinterpret_cast<const double2*>(dv.U);
    double2* dst = reinterpret_cast<double2*>(dv.U0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (5 * dv.nd > 2 * n2) dv.U0[5 * dv.nd - 1] = dv.U[5 * dv.nd - 1];
        s->time0 = s->time;
        s->n_steps0 = s->n_steps;
    }
}

static __global__ void k_clock(Dev dv)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    s->time += s->dt;
    s->n_steps += 1;
}

// --------------------------------------------------------------------------- time step
// PLENS::calc_time_step (dgsem/plens.cc:3810-3912): per-dof stable step, min over dofs. The
// plain form evaluates it in FP64 with the reference's expressions; the mixed form in FP32 (the
// step size is a CFL bound, not an accumulated quantity), from FP64 state and metrics converted on
// the integer pipes.
// the stable step of one dof (T: arithmetic type)
template <int P, class T>
__device__ __forceinline__ T dof_stable_step(const Dev& dv, const GasP& g, double N15, int N, int64_t dof, T Co)
{
    constexpr int P3 = P * P * P;
    const int64_t c = dof / P3;
    const T gm = to_real<T>(g.gamma);
    T cs[5];
    load_state<T>(dv, dof, cs);
    T a, vel[3];
    if constexpr (sizeof(T) == 8) {
        a = sqrt(gm * get_p(cs, gm) / cs[0]);
#pragma unroll
        for (int d = 0; d < 3; ++d) vel[d] = cs[1 + d] / cs[0];
    } else {
        a = sqrtf(__fdividef(gm * get_p(cs, gm), cs[0]));
        const T ri = __fdividef(1.0f, cs[0]);
#pragma unroll
        for (int d = 0; d < 3; ++d) vel[d] = cs[1 + d] * ri;
    }
    T adv[3];
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        T acc = T(0);
#pragma unroll
        for (int col = 0; col < 3; ++col) acc += metric<T>(dv.Jinv, dv.Jinvf, (col * 3 + row) * dv.nd + dof) * vel[col];
        adv[row] = acc;
    }
    T madv = adv[0];
    if (adv[1] > madv) madv = adv[1];
    if (adv[2] > madv) madv = adv[2];
    T mu = T(0);
    if (!g.inviscid) {
        if constexpr (sizeof(T) == 8) {
            const double Tk = get_e(cs) / (g.R / (g.gamma - 1));
            mu = g.const_visc ? g.mu0 : g.mu0 * pow(Tk / g.T0, 1.5) * (g.T0 + g.S) / (Tk + g.S);
        } else {
            const float Tk = __fdividef(get_e(cs) * to_real<T>(g.gamma - 1), to_real<T>(g.R));
            const float T0 = to_real<T>(g.T0), S = to_real<T>(g.S), x = __fdividef(Tk, T0);
            mu = g.const_visc ? to_real<T>(g.mu0) : to_real<T>(g.mu0) * x * sqrtf(x) * __fdividef(T0 + S, Tk + S);
        }
    }
    const T h = to_real<T>(dv.h_min[c]);
    return Co / (to_real<T>(N15) * (madv + a / h + (T)(N * N) * mu / (h * h * cs[0])));
}

// dofs per thread of the time-step kernel: two in the mixed form (their loads overlap)
template <class T> constexpr int kStepItems = (sizeof(T) == 4) ? 2 : 1;

template <int P, class T>
__global__ void __launch_bounds__(256) k_time_step(Dev dv, GasP g, double N15, int N)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    constexpr int K = kStepItems<T>;
    __shared__ T s_red[8];
    T local = T(1e6);
    const T Co = to_real<T>(s->courant);
    const int64_t base = blockIdx.x * (int64_t)blockDim.x * K + threadIdx.x;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int64_t dof = base + (int64_t)k * blockDim.x;
        if (dof < dv.nd) {
            const T cur = dof_stable_step<P, T>(dv, g, N15, N, dof, Co);
            if (cur < local) local = cur;
        }
    }
    // warp-shuffle min, then block min, then one atomic per block
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const T o = __shfl_xor_sync(0xffffffffu, local, off);
        if (o < local) local = o;
    }
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        T m = s_red[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (s_red[w] < m) m = s_red[w];
        atomicMin(&s->dtmin, ord_double(to_f64<T>(m)));
    }
}

// Local time stepping: the same per-dof bound, reduced per cell (one warp per cell) into
// dt_cell and over all cells into the global minimum (calc_time_step, dgsem/plens.cc:3836-3872).
template <int P, class T>
__global__ void __launch_bounds__(256) k_time_step_cells(Dev dv, GasP g, double N15, int N)
{
    constexpr int P3 = P * P * P;
    Scalars* s = dv.sc;
    if (!s->active) return;
    __shared__ double s_red[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t cell = blockIdx.x * 8ll + warp;
    const T Co = to_real<T>(s->courant);
    T local = T(1e6);
    if (cell < dv.nc)
        for (int l = lane; l < P3; l += 32) {
            const T cur = dof_stable_step<P, T>(dv, g, N15, N, cell * P3 + l, Co);
            if (cur < local) local = cur;
        }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const T o = __shfl_xor_sync(0xffffffffu, local, off);
        if (o < local) local = o;
    }
    const double cd = to_f64<T>(local);
    if (lane == 0) {
        if (cell < dv.nc) dv.dt_cell[cell] = cd;
        s_red[warp] = cd;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = s_red[0];
        for (int w = 1; w < 8; ++w)
            if (s_red[w] < m) m = s_red[w];
        atomicMin(&s->dtmin, ord_double(m));
    }
}

// loc_time_steps after the global reduction (dgsem/plens.cc:3880-3911): while local stepping is
// on (t > start), each cell's own step, optionally limited by factor x the unlimited steps of its
// interior-face neighbours (a periodic face is a boundary face: cell_nbr = -1) and by factor x
// the global step; otherwise the global step. All from the unclipped global step.
static __global__ void k_local_dt(Dev dv, int limit, double start_time, double nbr_factor, double global_factor)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= dv.nc) return;
    const double dtg = s->dt_update;
    double m = dtg;
    if (s->time > start_time) {
        m = dv.dt_cell[c];
        if (limit) {
            for (int f = 0; f < 6; ++f) {
                const int32_t nb = dv.cell_nbr[6 * c + f];
                if (nb >= 0) m = fmin(m, nbr_factor * dv.dt_cell[nb]);
            }
            m = fmin(m, global_factor * dtg);
        }
    }
    dv.dt_loc[c] = m;
}

// Courant number of the step from its expression of t (capped to 0.9 when >= 1,
// dgsem/plens.cc:3815-3823).
static __global__ void k_courant(Dev dv, int expr_courant)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    double Co = eval_expr(dv, expr_courant, 0, 0, 0, s->time);
    if (Co >= 1) Co = 0.9;
    s->courant = Co;
}

// ------------------------------------------------------------------------------- blender
// calc_blender's first half + BlenderCalculator::get_blender / get_trouble
// (dgsem/plens.cc:2858-2924, dgsem/blender_calculator.cc:123-177, 277-303), with
// assert_positivity (dgsem/plens.cc:2531-2546) fused in. The modal transform and the mode
// energies run in T (FP64 in the plain form and for the learned sensor's judge, FP32 in the
// mixed form); the positivity check and alpha are FP64.
// One tile of CPB cells (blk) of the blender; every thread of the block calls it.
template <int P, class T>
__device__ __forceinline__ void blender_tile(const int64_t blk, const Dev& dv, const Ops& ops, const GasP& g,
                                             const BlendP& bp, Scalars* s, const bool masked)
{
    using CB = CellBlock<P>;
    constexpr int P2 = CB::P2, P3 = CB::P3, CPB = CB::CPB, N = P - 1;
    __shared__ T sA[CPB][P3];
    __shared__ T sB[CPB][P3];
    if (masked) {  // learned sensor: only the cells the judge handed back to this indicator
        bool any = false;
#pragma unroll
        for (int q = 0; q < CPB; ++q) {
            const int64_t cq = blk * CPB + q;
            any |= (cq < dv.nc) && bp.mask[cq];
        }
        if (!any) return;
    }
    const int tid = threadIdx.x, cl = tid / P3, node = tid - cl * P3;
    const int64_t cell = blk * CPB + cl;
    const bool valid = (cl < CPB) && (cell < dv.nc) && (!masked || bp.mask[cell]);
    const int i = node % P, j = (node / P) % P, k = node / P2;
    if (valid) {
        const int64_t dof = cell * P3 + node;
        if constexpr (sizeof(T) == 8) {
            double c[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) c[v] = dv.U[v * dv.nd + dof];
            if (!(c[0] > 0) || !(get_e(c) > 0)) {
                atomicMin(&s->bad_dof, (long long)dof);
                s->err = PLENS_GPU_E_POSITIVITY;
            }
            const double p = get_p(c, g.gamma);
            sA[cl][node] = (bp.var == 2) ? c[0] : (bp.var == 1) ? p : p * c[0];
        } else {
            T cf[5];
            load_state<T>(dv, dof, cf);
            if (!positive_dof_screened(dv, dof, cf)) {
                atomicMin(&s->bad_dof, (long long)dof);
                s->err = PLENS_GPU_E_POSITIVITY;
            }
            const T p = get_p(cf, f64_to_f32(g.gamma));
            sA[cl][node] = (bp.var == 2) ? cf[0] : (bp.var == 1) ? p : p * cf[0];
        }
    }
    __syncthreads();
    // separable nodal -> modal transform: x, then y, then z
    if (valid) {
        T acc = 0;
#pragma unroll
        for (int m = 0; m < P; ++m) acc += opC1<T>(ops, i * P + m) * sA[cl][m + P * j + P2 * k];
        sB[cl][node] = acc;
    }
    __syncthreads();
    if (valid) {
        T acc = 0;
#pragma unroll
        for (int m = 0; m < P; ++m) acc += opC1<T>(ops, j * P + m) * sB[cl][i + P * m + P2 * k];
        sA[cl][node] = acc;
    }
    __syncthreads();
    if (valid) {
        T acc = 0;
#pragma unroll
        for (int m = 0; m < P; ++m) acc += opC1<T>(ops, k * P + m) * sA[cl][i + P * j + P2 * m];
        sB[cl][node] = acc;
    }
    __syncthreads();
    if constexpr (sizeof(T) == 4) {
        // mixed form: one warp per cell sums the mode energies (and the TV-filter statistics)
        // with shuffles; lane 0 evaluates alpha in FP32
        constexpr int NW = CB::THREADS / 32;
        const int warp = tid >> 5, lane = tid & 31;
        for (int q = warp; q < CPB; q += NW) {
            const int64_t cq = blk * CPB + q;
            if (cq >= dv.nc || (masked && !bp.mask[cq])) continue;
            float e0 = 0, e1 = 0, e2 = 0, asum = 0, ub = 0, tl = 0;
            for (int n = lane; n < P3; n += 32) {
                const float md = sB[q][n];
                const int mi = n % P, mj = (n / P) % P, mk = n / P2;
                const float e = md * md;
                e0 += e;
                if (mi < N && mj < N && mk < N) e1 += e;
                if (mi < N - 1 && mj < N - 1 && mk < N - 1) e2 += e;
                if (bp.do_filter) {
                    const float t = fabsf(md);
                    asum += t;
                    const float x = t * (ops.ftv[mi] + ops.ftv[mj] + ops.ftv[mk]);
                    ub += x;
                    if (mi <= 1 && mj <= 1 && mk <= 1) tl += x;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                e0 += __shfl_xor_sync(0xffffffffu, e0, off);
                e1 += __shfl_xor_sync(0xffffffffu, e1, off);
                e2 += __shfl_xor_sync(0xffffffffu, e2, off);
                if (bp.do_filter) {
                    asum += __shfl_xor_sync(0xffffffffu, asum, off);
                    ub += __shfl_xor_sync(0xffffffffu, ub, off);
                    tl += __shfl_xor_sync(0xffffffffu, tl, off);
                }
            }
            if (lane == 0) {
                float trouble = 1.0f - __fdividef(e1, e0);
                if (N > 2) {
                    const float t2 = 1.0f - __fdividef(e2, e1);
                    if (t2 > trouble) trouble = t2;
                }
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
                if (dv.cell_wall[cq]) {
                    const double wl = eval_expr(dv, bp.expr_wall, 0, 0, 0, s->time);
                    ad = (wl > ad) ? wl : ad;
                }
                dv.alpha_raw[cq] = ad;
                if (bp.do_filter) {
                    dv.tvstat[cq] = f32_to_f64(asum);
                    dv.tvstat[dv.nc + cq] = f32_to_f64(ub);
                    dv.tvstat[2 * dv.nc + cq] = f32_to_f64(tl);
                }
            }
        }
        return;
    }
    if (valid && node == 0) {
        // sums in mode-index order, as the reference's loops over the mode index sets
        T et = 0, e1 = 0, e2 = 0;
        double asum = 0, ub = 0, tl = 0;
        for (int m = 0; m < P3; ++m) {
            const T md = sB[cl][m];
            const int mi = m % P, mj = (m / P) % P, mk = m / P2;
            et += md * md;
            if (mi < N && mj < N && mk < N) e1 += md * md;
            if (mi < N - 1 && mj < N - 1 && mk < N - 1) e2 += md * md;
            if (bp.do_filter) {
                const double t = fabs((double)md);
                asum += t;
                const double x = t * (ops.tv[mi] + ops.tv[mj] + ops.tv[mk]);
                ub += x;
                if (mi <= 1 && mj <= 1 && mk <= 1) tl += x;
            }
        }
        double trouble = 1 - (double)(e1 / et);
        if (N > 2) {
            const double t2 = 1 - (double)(e2 / e1);
            if (t2 > trouble) trouble = t2;
        }
        double alpha;
        if (bp.func == 0) {
            const double at = 1 / (1 + exp(-bp.sharp * (trouble / bp.thr - 1)));
            alpha = (at < bp.amin) ? 0.0 : (at < bp.amax ? at : bp.amax);
        } else {
            const double at = trouble / bp.thr;
            alpha = (at > 1) ? 1.0 : at;
        }
        if (dv.cell_wall[cell]) {
            const double wl = eval_expr(dv, bp.expr_wall, 0, 0, 0, s->time);
            alpha = (wl > alpha) ? wl : alpha;
        }
        dv.alpha_raw[cell] = alpha;
        if (bp.do_filter) {
            dv.tvstat[cell] = asum;
            dv.tvstat[dv.nc + cell] = ub;
            dv.tvstat[2 * dv.nc + cell] = tl;
        }
    }
}

template <int P, class T>
__global__ void __launch_bounds__(CellBlock<P>::THREADS) k_blender(Dev dv, Ops ops, GasP g, BlendP bp)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    if (bp.gate && !s->sensor_fallback && !bp.mask) return;
    const bool masked = bp.mask && !s->sensor_fallback;
    const int64_t nblk = (dv.nc + CellBlock<P>::CPB - 1) / CellBlock<P>::CPB;
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        blender_tile<P, T>(blk, dv, ops, g, bp, s, masked);
        __syncthreads();  // shared tiles are reused by the next iteration
    }
}

// the rest of the smoothing of one cell after the neighbour max: TV filter, alpha, alpha_d
__device__ __forceinline__ void smooth_finish(const Dev& dv, const BlendP& bp, Scalars* s, int64_t c, double& a)
{
    if (bp.do_filter && !(a > bp.amin)) {
        const double asum = dv.tvstat[c], ub = dv.tvstat[dv.nc + c], tl = dv.tvstat[2 * dv.nc + c];
        if (!(ub < 1e-2 * asum)) a = a + (bp.amax - a) * (1 - tl / ub);
    }
    dv.alpha[c] = a;
    const double* x = dv.center + 3 * c;
    dv.alpha_d[c] = (eval_expr(dv, bp.expr_vis, x[0], x[1], x[2], s->time) > 0) ? ((1.0 < a / bp.amax) ? 1.0 : a / bp.amax) : 0.0;
}

constexpr int kSmoothThreads = 128;  // cells per block of k_alpha_smooth and k_lo_list (four warps)

// neighbour smoothing over interior faces against the pre-smoothing values, optional TV filter
// and alpha_d (dgsem/plens.cc:2926-2961, blender_calculator.cc:196-259); kSmoothThreads cells per
// block. Mixed forms: each block also counts its troubled cells (alpha > 0) for the compacted list.
static __global__ void __launch_bounds__(kSmoothThreads) k_alpha_smooth(Dev dv, BlendP bp)
{
    Scalars* s = dv.sc;
    if (!s->active) return;
    if (bp.gate && !s->sensor_fallback) return;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool troubled = false;
    if (c < dv.nc) {
        double a = dv.alpha_raw[c];
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const int32_t nb = dv.cell_nbr[6 * c + f];
            if (nb < 0) continue;
            const double h = 0.5 * dv.alpha_raw[nb];
            a = (h > a) ? h : a;
        }
        smooth_finish(dv, bp, s, c, a);
        troubled = stored_gt0<float>(a);  // the volume kernel's test of the stored alpha
    }
    if (dv.lo_blk) {
        const unsigned m = __ballot_sync(0xffffffffu, troubled);
        if ((threadIdx.x & 31) == 0) dv.lo_mask[4 * blockIdx.x + (threadIdx.x >> 5)] = m;
        const int n = __syncthreads_count(troubled ? 1 : 0);
        if (threadIdx.x == 0) dv.lo_blk[blockIdx.x] = n;
    }
}

// --------------------------------------------------------------------------- BC ghosts
// get_ghost_stage{1,2,3} of the BCs:: classes (IBCs/*.cc). Prescribed states are formed in double.
template <class T>
__device__ __forceinline__ void prim_to_cons_d(double rho, const double v[3], double p, double gma, T out[5])
{
    double c4 = p / (gma - 1);
    double c[5];
    c[0] = rho;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        c[1 + d] = rho * v[d];
        c4 += 0.5 * rho * v[d] * v[d];
    }
    c[4] = c4;
#pragma unroll
    for (int v2 = 0; v2 < 5; ++v2) out[v2] = to_real<T>(c[v2]);
}

template <class T>
__device__ __forceinline__ void prim_to_cons_t(T rho, const T v[3], T p, T gma, T c[5])
{
    c[0] = rho;
    T c4 = p / (gma - 1);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        c[1 + d] = rho * v[d];
        c4 += T(0.5) * rho * v[d] * v[d];
    }
    c[4] = c4;
}

template <class T>
__device__ __forceinline__ void bc_ghost(int stage, const Dev& dv, const GasP& g, const plens_bc_desc& b,
                         const T c[5], const T av[9], const T n[3], const double* xyz, double t,
                         int64_t partner_dof, T cg[5], T ag[9])
{
    const T gm = to_real<T>(g.gamma);
#pragma unroll
    for (int v = 0; v < 9; ++v) ag[v] = av[v];
    switch (b.type) {
    case PLENS_BC_PERIODIC:
#pragma unroll
        for (int v = 0; v < 5; ++v) cg[v] = (sizeof(T) == 8) ? (T)dv.U[v * dv.nd + partner_dof] : (T)dv.Uf[v * dv.nd + partner_dof];
        if (stage == 3)
#pragma unroll
            for (int v = 0; v < 9; ++v) ag[v] = as_real<T>(dv.avars)[v * dv.nd + partner_dof];
        return;
    case PLENS_BC_OUTFLOW: {
#pragma unroll
        for (int v = 0; v < 5; ++v) cg[v] = c[v];
        if (stage == 2 && !g.inviscid) {
            const T ri = T(1) / c[0];
            T sp = (c[1] * c[1]) * (ri * ri);
            sp += (c[2] * c[2]) * (ri * ri);
            sp += (c[3] * c[3]) * (ri * ri);
            const T pin = get_p(c, gm);
            const T M = dsqrt(sp) / dsqrt(gm * pin / c[0]);
            if (!(M >= T(1))) cg[4] += T(2) * (to_real<T>(b.p) - pin) / (gm - 1);
        }
        return;
    }
    case PLENS_BC_UNIFORM_INFLOW:
        if (stage == 2) {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = to_real<T>(b.cons[v]);
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = T(2) * to_real<T>(b.cons[v]) - c[v];
        }
        return;
    case PLENS_BC_VARYING_INFLOW: {
        const double p = eval_expr(dv, b.expr_p, xyz[0], xyz[1], xyz[2], t);
        const double Tt = eval_expr(dv, b.expr_T, xyz[0], xyz[1], xyz[2], t);
        double vel[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) vel[d] = eval_expr(dv, b.expr_vel[d], xyz[0], xyz[1], xyz[2], t);
        T cp[5];
        prim_to_cons_d(p / (g.R * Tt), vel, p, g.gamma, cp);
        if (stage == 2) {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = cp[v];
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = T(2) * cp[v] - c[v];
        }
        return;
    }
    case PLENS_BC_UNIFORM_TEMP_WALL:
    case PLENS_BC_INSULATED_WALL: {
        const T vw[3] = {to_real<T>(b.vel[0]), to_real<T>(b.vel[1]), to_real<T>(b.vel[2])};
        if (stage == 2) {
            cg[0] = c[0];
            cg[4] = c[4];
            if (g.inviscid) {
                T sr[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) sr[d] = c[1 + d] - c[0] * vw[d];
                T nsm = sr[0] * n[0];
                nsm += sr[1] * n[1];
                nsm += sr[2] * n[2];
#pragma unroll
                for (int d = 0; d < 3; ++d) cg[1 + d] = c[1 + d] - T(2) * nsm * n[d];
            } else {
#pragma unroll
                for (int d = 0; d < 3; ++d) cg[1 + d] = T(2) * c[0] * vw[d] - c[1 + d];
            }
            return;
        }
        const T pin = get_p(c, gm);
        const T rho_pr = (b.type == PLENS_BC_UNIFORM_TEMP_WALL) ? pin / (to_real<T>(g.R) * to_real<T>(b.T)) : c[0];
        T cp[5];
        prim_to_cons_t(rho_pr, vw, pin, gm, cp);
#pragma unroll
        for (int v = 0; v < 5; ++v) cg[v] = T(2) * cp[v] - c[v];
        if (stage == 3 && b.type == PLENS_BC_INSULATED_WALL) {
            T nh = av[6] * n[0];
            nh += av[7] * n[1];
            nh += av[8] * n[2];
#pragma unroll
            for (int d = 0; d < 3; ++d) ag[6 + d] = av[6 + d] - T(2) * nh * n[d];
        }
        return;
    }
    case PLENS_BC_SYMMETRY:
    case PLENS_BC_EMPTY: {
        if (stage == 2 && b.type == PLENS_BC_SYMMETRY) {
            cg[0] = c[0];
            cg[4] = c[4];
            T nsm = c[1] * n[0];
            nsm += c[2] * n[1];
            nsm += c[3] * n[2];
#pragma unroll
            for (int d = 0; d < 3; ++d) cg[1 + d] = c[1 + d] - T(2) * nsm * n[d];
            return;
        }
        T vin[3], vpr[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) vin[d] = c[1 + d] / c[0];
        T nv = vin[0] * n[0];
        nv += vin[1] * n[1];
        nv += vin[2] * n[2];
#pragma unroll
        for (int d = 0; d < 3; ++d) vpr[d] = vin[d] - nv * n[d];
        T cp[5];
        prim_to_cons_t(c[0], vpr, get_p(c, gm), gm, cp);
        if (stage == 2) {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = cp[v];
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = T(2) * cp[v] - c[v];
        }
        return;
    }
    case PLENS_BC_ZPG_INFLOW: {
        const T vw[3] = {to_real<T>(b.vel[0]), to_real<T>(b.vel[1]), to_real<T>(b.vel[2])};
        T cp[5];
        prim_to_cons_t(c[0], vw, get_p(c, gm), gm, cp);
        if (stage == 2) {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = cp[v];
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) cg[v] = T(2) * cp[v] - c[v];
        }
        return;
    }
    default:  // free
#pragma unroll
        for (int v = 0; v < 5; ++v) cg[v] = c[v];
        return;
    }
}

// -------------------------------------------------------------------------- surface flux
// PLENS::calc_surf_flux (dgsem/plens.cc:1717-1913) for one stage: one thread per face dof of a
// face task. Interior faces are computed once and written to both sides (neighbour sign +1 in
// stage 1, -1 in stages 2 and 3); boundary faces (periodic included) once per side.
template <int P, class T, int STAGE>
__global__ void __launch_bounds__(128, (sizeof(T) == 4 ? 10 : 1)) k_surface(Dev dv, GasP g, double* out)
{
    constexpr int P2 = P * P;
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= dv.ntask * P2) return;
    const int64_t ti = idx / P2;
    const int q = (int)(idx - ti * P2);
    const int bc = dv.ft_bc[ti];
    // precomputed dofs of both sides: the loads of the two states do not wait on each other
    const int64_t gd = dv.fd_own[idx], gdn = dv.fd_nbr[idx];
    const T gm = to_real<T>(g.gamma);
    const T* avs = as_real<T>(dv.avars);
    T cs[5], av[9] = {}, n[3], c2[5], a2[9] = {};
    load_state<T>(dv, gd, cs);
    if (gdn >= 0) load_state<T>(dv, gdn, c2);
    if (STAGE == 3) {
#pragma unroll
        for (int v = 0; v < 9; ++v) av[v] = avs[v * dv.nd + gd];
        if (gdn >= 0)
#pragma unroll
            for (int v = 0; v < 9; ++v) a2[v] = avs[v * dv.nd + gdn];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) n[d] = to_real<T>(dv.ft_normal[idx * 3 + d]);
    T fb = T(0);
    // the flux blender enters the Chandrashekhar and Rusanov-blended schemes only
    if (STAGE == 2 && (g.isf == PLENS_ISF_CHANDRASHEKHAR || g.isf == PLENS_ISF_RUSANOV_HLLC ||
                       g.isf == PLENS_ISF_RUSANOV_AUSM_PLUS_UP)) {
        const int64_t c = dv.ft_cell[ti];
        if constexpr (sizeof(T) == 8) {
            double a = (bc >= 0) ? dv.alpha[c] : 0.5 * (dv.alpha[c] + dv.alpha[dv.ft_nbr_cell[ti]]);
            fb = (a <= 0) ? 0.0 : (a <= 1 ? a : 1.0);
        } else {
            float a = f64_to_f32(dv.alpha[c]);
            if (bc < 0) a = 0.5f * (a + f64_to_f32(dv.alpha[dv.ft_nbr_cell[ti]]));
            fb = (a <= 0.0f) ? 0.0f : (a <= 1.0f ? a : 1.0f);
        }
    }
    const int64_t slot_nb = dv.fs_nbr[idx];
    if (bc >= 0) {
        const plens_bc_desc& b = dv.bcs[bc];
        // periodic: the partner's state (and auxiliary variables) loaded above is the ghost
        if (b.type != PLENS_BC_PERIODIC)
            bc_ghost<T>(STAGE, dv, g, b, cs, av, n, dv.ft_xyz + idx * 3, s->time, -1, c2, a2);
    }
    T fl[5];
    if (STAGE == 1) {
#pragma unroll
        for (int v = 0; v < 5; ++v) fl[v] = T(0.5) * (cs[v] + c2[v]);
    } else if (STAGE == 2) {
        if constexpr (sizeof(T) == 4) inv_surf_flux_mx(cs, c2, n, gm, g.isf, fb, fl);
        else inv_surf_flux(cs, c2, n, gm, g.isf, fb, fl);
    } else {
        T f1[5], f2[5];
        dif_flux(cs, av, n, f1);
        dif_flux(c2, a2, n, f2);
#pragma unroll
        for (int v = 0; v < 5; ++v) fl[v] = T(0.5) * (f1[v] + f2[v]);
    }
    const int64_t slot = dv.fs_own[idx];
    T* o = as_real<T>(out);
#pragma unroll
    for (int v = 0; v < 5; ++v) o[v * dv.nslot + slot] = fl[v];
    if (slot_nb >= 0) {
        const T sg = (STAGE == 1) ? T(1) : T(-1);
#pragma unroll
        for (int v = 0; v < 5; ++v) o[v * dv.nslot + slot_nb] = sg * fl[v];
    }
}

// ----------------------------------------------------------------------- auxiliary variables
// PLENS::calc_aux_vars + calc_cell_evar_grad (dgsem/plens.cc:2593-2748, 2294-2405): BR1 lifting
// of the entropy variables, then the stress tensor and heat flux scaled by mu and k.
template <int P, class T>
__global__ void __launch_bounds__(CellBlock<P>::THREADS, (sizeof(T) == 4 && P == 4) ? 8 : 1) k_aux(Dev dv, Ops ops, GasP g)
{
    using CB = CellBlock<P>;
    constexpr int P2 = CB::P2, P3 = CB::P3, CPB = CB::CPB, N = P - 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sE = reinterpret_cast<T*>(smem_raw);        // [CPB][5][P3]
    T* sJa = sE + CPB * 5 * P3;                     // [CPB][9][P3]
    T* sEf = sJa + CPB * 9 * P3;                    // [CPB][6][5][P2]
    // D in shared memory: the lanes of a warp read different entries of it, which the constant
    // cache would serve one address at a time
    __shared__ T sD[P * P];
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int tid = threadIdx.x, cl = tid / P3, node = tid - cl * P3;
    const int64_t cell = (int64_t)blockIdx.x * CPB + cl;
    const bool valid = (cl < CPB) && (cell < dv.nc);
    const T gm = to_real<T>(g.gamma);
    for (int k = tid; k < P * P; k += blockDim.x) sD[k] = opD<T>(ops, k);
    T cd[5] = {1, 0, 0, 0, 1};  // the node's state in T (FP64 state, or its FP32 image)
    T ev[5] = {0, 0, 0, 0, 0};   // and its entropy variables
    T dj = T(1);                  // and det J
    if (valid) {
        // every load of the thread first (state, metric terms, det J, its face slots), then the
        // arithmetic: one memory latency per block instead of one per group of loads
        constexpr int NS = (6 * P2 + P3 - 1) / P3;  // face slots per thread
        const int64_t dof = cell * P3 + node;
        T ja[9], fc[NS][5];
        load_state<T>(dv, dof, cd);
#pragma unroll
        for (int m = 0; m < 9; ++m) ja[m] = metric<T>(dv.Ja, dv.Jaf, m * dv.nd + dof);
        dj = metric<T>(dv.detJ, dv.detJf, dof);
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const int sl = node + k * P3;
            if (sl < 6 * P2)
#pragma unroll
                for (int v = 0; v < 5; ++v) fc[k][v] = as_real<T>(dv.sf)[v * dv.nslot + cell * 6 * P2 + sl];
        }
        cons_to_entropy(cd, gm, ev);
#pragma unroll
        for (int v = 0; v < 5; ++v) sE[(cl * 5 + v) * P3 + node] = ev[v];
#pragma unroll
        for (int m = 0; m < 9; ++m) sJa[(cl * 9 + m) * P3 + node] = ja[m];
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const int sl = node + k * P3;
            if (sl < 6 * P2) {
                T fe[5];
                cons_to_entropy(fc[k], gm, fe);
#pragma unroll
                for (int v = 0; v < 5; ++v) sEf[((cl * 6 + sl / P2) * 5 + v) * P2 + (sl % P2)] = fe[v];
            }
        }
    }
    __syncthreads();
    if (!valid) return;
    const int ti[3] = {node % P, (node / P) % P, node / P2};
    const T* E = sE + cl * 5 * P3;
    const T* J = sJa + cl * 9 * P3;
    // volume terms: sum_m sum_md D_(i,m) (E Ja_md,gd)_m, each line node's E and Ja row loaded once
    // for the three gradient directions; per direction gd the terms add in the order m, md
    T acc[3][5];
#pragma unroll
    for (int gd = 0; gd < 3; ++gd)
#pragma unroll
        for (int v = 0; v < 5; ++v) acc[gd][v] = T(0);
#pragma unroll
    for (int m = 0; m < P; ++m) {
#pragma unroll
        for (int md = 0; md < 3; ++md) {
            const int lo = (md == 0) ? m + P * ti[1] + P2 * ti[2] : (md == 1) ? ti[0] + P * m + P2 * ti[2] : ti[0] + P * ti[1] + P2 * m;
            T de[5], jc[3];
            const T dvl = sD[ti[md] * P + m];
#pragma unroll
            for (int v = 0; v < 5; ++v) de[v] = dvl * E[v * P3 + lo];
#pragma unroll
            for (int gd = 0; gd < 3; ++gd) jc[gd] = J[(md * 3 + gd) * P3 + lo];
#pragma unroll
            for (int gd = 0; gd < 3; ++gd)
#pragma unroll
                for (int v = 0; v < 5; ++v) acc[gd][v] += de[v] * jc[gd];
        }
    }
    const T jinv = fdiv(T(1.0), dj);
    T grad[3][5];
    if constexpr (sizeof(T) == 4) {
        // FP32 (mixed forms): a face's term for direction gd is -sign Ja_gd (E_face - E) / w, the
        // difference formed once per face and variable for the three directions
#pragma unroll
        for (int sd = 0; sd < 3; ++sd) {
#pragma unroll
            for (int lr = 0; lr < 2; ++lr) {
                if (ti[sd] != (lr ? N : 0)) continue;
                const int f = 2 * sd + lr;
                const int q = (sd == 0) ? ti[1] + P * ti[2] : (sd == 1) ? ti[0] + P * ti[2] : ti[0] + P * ti[1];
                const T sw = __fdividef(lr ? 1.0f : -1.0f, opW<T>(ops, lr * N));
                T de[5], js[3];
#pragma unroll
                for (int v = 0; v < 5; ++v) de[v] = sEf[((cl * 6 + f) * 5 + v) * P2 + q] - ev[v];
#pragma unroll
                for (int gd = 0; gd < 3; ++gd) js[gd] = J[(sd * 3 + gd) * P3 + node] * sw;
#pragma unroll
                for (int gd = 0; gd < 3; ++gd)
#pragma unroll
                    for (int v = 0; v < 5; ++v) acc[gd][v] += js[gd] * de[v];
            }
        }
#pragma unroll
        for (int gd = 0; gd < 3; ++gd)
#pragma unroll
            for (int v = 0; v < 5; ++v) grad[gd][v] = acc[gd][v] * jinv;
    } else {
        // FP64: the reference's order, -sign (F_face Ja - F_in Ja) / w (bit-level parity with the
        // oracle in the strongly stretched wall cells, where the terms cancel)
#pragma unroll
        for (int gd = 0; gd < 3; ++gd) {
#pragma unroll
            for (int sd = 0; sd < 3; ++sd) {
#pragma unroll
                for (int lr = 0; lr < 2; ++lr) {
                    if (ti[sd] != (lr ? N : 0)) continue;
                    const int f = 2 * sd + lr;
                    const int q = (sd == 0) ? ti[1] + P * ti[2] : (sd == 1) ? ti[0] + P * ti[2] : ti[0] + P * ti[1];
                    const T jc = J[(sd * 3 + gd) * P3 + node];
                    const T sgn = lr ? T(-1) : T(1);
                    const T wend = opW<T>(ops, lr * N);
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        const T fin = ev[v] * jc;
                        const T fsu = sEf[((cl * 6 + f) * 5 + v) * P2 + q] * jc;
                        acc[gd][v] -= fdiv(sgn * (fsu - fin), wend);
                    }
                }
            }
#pragma unroll
            for (int v = 0; v < 5; ++v) grad[gd][v] = acc[gd][v] * jinv;
        }
    }
    const int64_t dof = cell * P3 + node;
    const T* et = ev;
    T vg[3][3];
    if constexpr (sizeof(T) == 4) {
        const T ri = __fdividef(1.0f, et[4]);  // one reciprocal for the eighteen divisions by e4
#pragma unroll
        for (int vd = 0; vd < 3; ++vd)
#pragma unroll
            for (int gd = 0; gd < 3; ++gd) vg[vd][gd] = (et[1 + vd] * grad[gd][4] * ri - grad[gd][1 + vd]) * ri;
    } else {
#pragma unroll
        for (int vd = 0; vd < 3; ++vd)
#pragma unroll
            for (int gd = 0; gd < 3; ++gd) vg[vd][gd] = (et[1 + vd] * grad[gd][4] / et[4] - grad[gd][1 + vd]) / et[4];
    }
    const T tr = vg[0][0] + vg[1][1] + vg[2][2];
    // mu and k (NavierStokes::get_mu / get_k, h:348-360): FP64 from the FP64 state in the plain
    // form, FP32 in the mixed form
    T mu, kk;
    if constexpr (sizeof(T) == 8) {
        const double e = get_e(cd);
        const double Tk = e / (g.R / (g.gamma - 1));
        mu = g.const_visc ? g.mu0 : g.mu0 * pow(Tk / g.T0, 1.5) * (g.T0 + g.S) / (Tk + g.S);
        kk = mu * g.R * g.gamma / ((g.gamma - 1) * g.Pr);
    } else {
        const T* c = cd;
        const float Rg = to_real<T>(g.R), gm1 = to_real<T>(g.gamma - 1);
        const float Tk = __fdividef(get_e(c) * gm1, Rg);
        const float T0 = to_real<T>(g.T0), S = to_real<T>(g.S), x = __fdividef(Tk, T0);
        mu = g.const_visc ? to_real<T>(g.mu0) : to_real<T>(g.mu0) * x * sqrtf(x) * __fdividef(T0 + S, Tk + S);
        kk = mu * __fdividef(Rg * gm, gm1 * to_real<T>(g.Pr));
    }
    T tau[6];
    int sid = 0;
#pragma unroll
    for (int row = 0; row < 3; ++row)
#pragma unroll
        for (int col = row; col < 3; ++col) {
            tau[sid] = (col == row) ? vg[row][col] + vg[col][row] - T(2.0) / T(3) * tr : vg[row][col] + vg[col][row];
            ++sid;
        }
#pragma unroll
    for (int v = 0; v < 6; ++v) as_real<T>(dv.avars)[v * dv.nd + dof] = tau[v] * mu;
#pragma unroll
    for (int gd = 0; gd < 3; ++gd) {
        const T tg = grad[gd][4] / (et[4] * et[4] * to_real<T>(g.R));
        as_real<T>(dv.avars)[(6 + gd) * dv.nd + dof] = (-tg) * kk;
    }
}

// ------------------------------------------------------------------------------ volume
// One RHS of a cell: calc_cell_ho_inv_residual (dgsem/plens.cc:3153-3275), calc_cell_ho_dif_residual
// (3283-3413), calc_cell_lo_inv_residual (3469-3583), the blend of calc_rhs (3753-3775), and --
// when stepping -- multiply_time_step_to_rhs (3925-3940) and the register update of update_rk4 /
// update_rk3 (4353-4400, 4433-4472). The two-point volume fluxes are evaluated once per node pair
// of a line (F_im = F_mi) by one thread per line; per-direction partial sums live in shared memory
// owned by exactly one thread, so the accumulation is deterministic.
template <int P, class T>
struct VolSmem {
    static constexpr int P3 = P * P * P;
    static constexpr int CPB = CellBlock<P>::CPB;
    // rho, 1/rho, v0, v1, v2, p, beta (+ ln rho, ln beta, |v|^2 in the mixed form)
    static constexpr int NQ = (sizeof(T) == 4) ? 10 : 7;
    static constexpr size_t bytes(bool visc)
    {
        return sizeof(T) * (size_t)CPB * P3 * (NQ + 5 + 9 + 15 + (visc ? 9 : 0) + 1);
    }
};

template <int P, class T, bool VISC>
__global__ void __launch_bounds__(CellBlock<P>::THREADS, (sizeof(T) == 4 ? 5 : 1)) k_volume(Dev dv, Ops ops, GasP g, StageArgs sa)
{
    using CB = CellBlock<P>;
    constexpr int P2 = CB::P2, P3 = CB::P3, CPB = CB::CPB, N = P - 1, NQ = VolSmem<P, T>::NQ;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sQ = reinterpret_cast<T*>(smem_raw);   // [CPB][NQ][P3]
    T* sC = sQ + CPB * NQ * P3;               // [CPB][5][P3]
    T* sJ = sC + CPB * 5 * P3;                // [CPB][9][P3]
    T* sAcc = sJ + CPB * 9 * P3;              // [CPB][3][5][P3]
    T* sAv = sAcc + CPB * 15 * P3;            // [CPB][9][P3] (viscous)
    T* sNorm = sAv + (VISC ? CPB * 9 * P3 : 0);  // [CPB][P3] scratch
    (void)sNorm;
    Scalars* s = dv.sc;
    // a positivity failure earlier in this step stops the updates: the state stays that of the
    // RHS that failed, as the reference exits there (assert_positivity, dgsem/plens.cc:2531-2546)
    if (!s->active || s->err) return;
    const int tid = threadIdx.x, cl = tid / P3, node = tid - cl * P3;
    const int64_t cell = (int64_t)blockIdx.x * CPB + cl;
    const bool valid = (cl < CPB) && (cell < dv.nc);
    const T gm = to_real<T>(g.gamma);
    T* Q = sQ + cl * NQ * P3;
    T* Cc = sC + cl * 5 * P3;
    T* J = sJ + cl * 9 * P3;
    T* Acc = sAcc + cl * 15 * P3;
    T* Av = sAv + cl * 9 * P3;
    const int64_t dof = cell * P3 + node;
    // FP64 state of the node: kept in registers by the plain form; the mixed form reads it again
    // for the update (an L2 hit), which frees ten registers through the flux phases
    double ud[5] = {0, 0, 0, 0, 0};
    if (valid) {
        T c[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const double u = dv.U[v * dv.nd + dof];
            if constexpr (sizeof(T) == 8) ud[v] = u;
            c[v] = to_real<T>(u);
            Cc[v * P3 + node] = c[v];
        }
        // per-node quantities with the reference's own expressions
        const T p = get_p(c, gm);
        const T ri = T(1) / c[0];
        Q[0 * P3 + node] = c[0];
        Q[1 * P3 + node] = ri;
        Q[2 * P3 + node] = c[1] * ri;
        Q[3 * P3 + node] = c[2] * ri;
        Q[4 * P3 + node] = c[3] * ri;
        Q[5 * P3 + node] = p;
        Q[6 * P3 + node] = T(0.5) * c[0] / p;
        if constexpr (sizeof(T) == 4) {
            Q[7 * P3 + node] = __logf(c[0]);
            Q[8 * P3 + node] = __logf(Q[6 * P3 + node]);
            Q[9 * P3 + node] = Q[2 * P3 + node] * Q[2 * P3 + node] + Q[3 * P3 + node] * Q[3 * P3 + node] +
                               Q[4 * P3 + node] * Q[4 * P3 + node];
        }
#pragma unroll
        for (int m = 0; m < 9; ++m) J[m * P3 + node] = metric<T>(dv.Ja, dv.Jaf, m * dv.nd + dof);
        if (VISC) {
#pragma unroll
            for (int m = 0; m < 9; ++m) Av[m * P3 + node] = as_real<T>(dv.avars)[m * dv.nd + dof];
        }
    }
    __syncthreads();
    const double alpha = valid ? dv.alpha[cell] : 0.0;
    const T alpha_t = to_real<T>(alpha);

    // ---- phase A: two-point volume fluxes per line
    bool fast_done = false;
    if constexpr (sizeof(T) == 4) {
        // mixed form, Chandrashekhar volume flux: unnormalised directions, per-node logarithms;
        // the diagonal term is kept at the two end nodes only (D_ii = 0 at interior GLL nodes)
        if (g.ivf == PLENS_IVF_CHANDRASHEKHAR) {
            fast_done = true;
            const float hg = __fdividef(0.5f, gm - 1.0f), gf = __fdividef(gm, gm - 1.0f);
            if (valid) {
                for (int task = node; task < 3 * P2; task += P3) {
                    const int dir = task / P2, line = task - dir * P2, la = line % P, lb = line / P;
                    float acc[P][5];
#pragma unroll
                    for (int i = 0; i < P; ++i)
#pragma unroll
                        for (int v = 0; v < 5; ++v) acc[i][v] = 0.0f;
#pragma unroll
                    for (int i = 0; i < P; ++i) {
                        const int ni = line_node<P>(dir, la, lb, i);
                        float qi[10];
#pragma unroll
                        for (int k = 0; k < 10; ++k) qi[k] = Q[k * P3 + ni];
                        const float ji[3] = {J[(dir * 3) * P3 + ni], J[(dir * 3 + 1) * P3 + ni], J[(dir * 3 + 2) * P3 + ni]};
                        if (i == 0 || i == N) {
                            float F[5];
                            chandrashekhar_same_f32(qi, ji, gf, F);
                            const float dd = opD2<float>(ops, i * P + i);
#pragma unroll
                            for (int v = 0; v < 5; ++v) acc[i][v] += dd * F[v];
                        }
#pragma unroll
                        for (int m = i + 1; m < P; ++m) {
                            const int nm = line_node<P>(dir, la, lb, m);
                            float qm[10];
#pragma unroll
                            for (int k = 0; k < 10; ++k) qm[k] = Q[k * P3 + nm];
                            const float nv[3] = {ji[0] + J[(dir * 3) * P3 + nm], ji[1] + J[(dir * 3 + 1) * P3 + nm],
                                                 ji[2] + J[(dir * 3 + 2) * P3 + nm]};
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
#pragma unroll
                    for (int i = 0; i < P; ++i) {
                        const int ni = line_node<P>(dir, la, lb, i);
#pragma unroll
                        for (int v = 0; v < 5; ++v) Acc[(dir * 5 + v) * P3 + ni] = acc[i][v];
                    }
                }
            }
        }
    }
    if (valid && !fast_done) {
        for (int task = node; task < 3 * P2; task += P3) {
            const int dir = task / P2, line = task - dir * P2, la = line % P, lb = line / P;
            T acc[P][5];
#pragma unroll
            for (int i = 0; i < P; ++i)
#pragma unroll
                for (int v = 0; v < 5; ++v) acc[i][v] = T(0);
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int ni = line_node<P>(dir, la, lb, i);
                T qi[7];
#pragma unroll
                for (int k = 0; k < 7; ++k) qi[k] = Q[k * P3 + ni];
                const T ci[5] = {Cc[ni], Cc[P3 + ni], Cc[2 * P3 + ni], Cc[3 * P3 + ni], Cc[4 * P3 + ni]};
                // diagonal term m = i (the pair flux of a state with itself)
                {
                    // 0.5*(Ja_i + Ja_i) = Ja_i exactly
                    const T nv[3] = {J[(dir * 3) * P3 + ni], J[(dir * 3 + 1) * P3 + ni], J[(dir * 3 + 2) * P3 + ni]};
                    T nn = nv[0] * nv[0];
                    nn += nv[1] * nv[1];
                    nn += nv[2] * nv[2];
                    nn = dsqrt(nn);
                    const T dn[3] = {fdiv(nv[0], nn), fdiv(nv[1], nn), fdiv(nv[2], nn)};
                    T F[5];
                    if (g.ivf == PLENS_IVF_CHANDRASHEKHAR) chandrashekhar_vol_same(qi, dn, gm, F);
                    else if (g.ivf == PLENS_IVF_KENNEDY_GRUBER) kennedy_gruber_vol(qi, qi, get_e(ci), get_e(ci), dn, gm, F);
                    else ismail_roe_vol(ci, ci, dn, gm, F);
                    const T dvn = opD2<T>(ops, i * P + i) * nn;
#pragma unroll
                    for (int v = 0; v < 5; ++v) acc[i][v] += dvn * F[v];
                }
#pragma unroll
                for (int m = i + 1; m < P; ++m) {
                    const int nm = line_node<P>(dir, la, lb, m);
                    T qm[7];
#pragma unroll
                    for (int k = 0; k < 7; ++k) qm[k] = Q[k * P3 + nm];
                    T nv[3];
#pragma unroll
                    for (int d = 0; d < 3; ++d) nv[d] = T(0.5) * (J[(dir * 3 + d) * P3 + ni] + J[(dir * 3 + d) * P3 + nm]);
                    T nn = nv[0] * nv[0];
                    nn += nv[1] * nv[1];
                    nn += nv[2] * nv[2];
                    nn = dsqrt(nn);
                    const T dn[3] = {fdiv(nv[0], nn), fdiv(nv[1], nn), fdiv(nv[2], nn)};
                    T F[5];
                    if (g.ivf == PLENS_IVF_CHANDRASHEKHAR) {
                        chandrashekhar_vol(qi, qm, dn, gm, F);
                    } else if (g.ivf == PLENS_IVF_KENNEDY_GRUBER) {
                        const T cm[5] = {Cc[nm], Cc[P3 + nm], Cc[2 * P3 + nm], Cc[3 * P3 + nm], Cc[4 * P3 + nm]};
                        kennedy_gruber_vol(qi, qm, get_e(ci), get_e(cm), dn, gm, F);
                    } else {
                        const T cm[5] = {Cc[nm], Cc[P3 + nm], Cc[2 * P3 + nm], Cc[3 * P3 + nm], Cc[4 * P3 + nm]};
                        ismail_roe_vol(ci, cm, dn, gm, F);
                    }
                    const T di = opD2<T>(ops, i * P + m) * nn, dm = opD2<T>(ops, m * P + i) * nn;
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        acc[i][v] += di * F[v];
                        acc[m][v] += dm * F[v];
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int ni = line_node<P>(dir, la, lb, i);
#pragma unroll
                for (int v = 0; v < 5; ++v) Acc[(dir * 5 + v) * P3 + ni] = acc[i][v];
            }
        }
    }
    __syncthreads();

    // ---- phase B: HO inviscid = volume + surface, scaled by 1/(-detJ)
    const int ti[3] = {node % P, (node / P) % P, node / P2};
    const T detJt = valid ? metric<T>(dv.detJ, dv.detJf, dof) : T(1);
    // MIXED form: the residual's parts stay unscaled FP32 sums, scaled by 1/detJ in FP64 below
    const bool u64 = sizeof(T) == 4 && sa.reg64;
    T ho[5] = {0, 0, 0, 0, 0};
    if (valid) {
#pragma unroll
        for (int v = 0; v < 5; ++v) ho[v] = Acc[v * P3 + node] + Acc[(5 + v) * P3 + node] + Acc[(10 + v) * P3 + node];
        const T ci[5] = {Cc[node], Cc[P3 + node], Cc[2 * P3 + node], Cc[3 * P3 + node], Cc[4 * P3 + node]};
#pragma unroll
        for (int sd = 0; sd < 3; ++sd) {
#pragma unroll
            for (int lr = 0; lr < 2; ++lr) {
                if (ti[sd] != (lr ? N : 0)) continue;
                const int f = 2 * sd + lr;
                const int q = (sd == 0) ? ti[1] + P * ti[2] : (sd == 1) ? ti[0] + P * ti[2] : ti[0] + P * ti[1];
                T dn[3] = {J[(sd * 3) * P3 + node], J[(sd * 3 + 1) * P3 + node], J[(sd * 3 + 2) * P3 + node]};
                T nn = dn[0] * dn[0];
                nn += dn[1] * dn[1];
                nn += dn[2] * dn[2];
                nn = dsqrt(nn);
#pragma unroll
                for (int d = 0; d < 3; ++d) dn[d] = fdiv(dn[d], nn);
                T fin[5];
                inv_flux(ci, dn, gm, fin);
                const T ss = lr ? T(-1) : T(1);
                const T wend = opW<T>(ops, lr * N);
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    const T fs = -ss * as_real<T>(dv.sf)[v * dv.nslot + (cell * 6 + f) * P2 + q];
                    ho[v] += fdiv(-ss * (fs - fin[v]) * nn, wend);
                }
            }
        }
        // the MIXED form scales the FP32 sums by 1/detJ in FP64 in phase D
        if (!u64) {
            const T js = fdiv(T(1), T(-1) * detJt);
#pragma unroll
            for (int v = 0; v < 5; ++v) ho[v] *= js;
        }
    }

    // ---- viscous HO residual: nodal viscous fluxes along each contravariant direction
    T hd[5] = {0, 0, 0, 0, 0};
    if (VISC) {
        __syncthreads();  // Acc is reused
        if (valid) {
            const T ci[5] = {Cc[node], Cc[P3 + node], Cc[2 * P3 + node], Cc[3 * P3 + node], Cc[4 * P3 + node]};
            T av[9];
#pragma unroll
            for (int m = 0; m < 9; ++m) av[m] = Av[m * P3 + node];
#pragma unroll
            for (int md = 0; md < 3; ++md) {
                T dn[3] = {J[(md * 3) * P3 + node], J[(md * 3 + 1) * P3 + node], J[(md * 3 + 2) * P3 + node]};
                T nn = dn[0] * dn[0];
                nn += dn[1] * dn[1];
                nn += dn[2] * dn[2];
                nn = dsqrt(nn);
#pragma unroll
                for (int d = 0; d < 3; ++d) dn[d] = fdiv(dn[d], nn);
                T F[5];
                dif_flux(ci, av, dn, F);
#pragma unroll
                for (int v = 0; v < 5; ++v) Acc[(md * 5 + v) * P3 + node] = F[v] * nn;
            }
        }
        __syncthreads();
        if (valid) {
            for (int m = 0; m < P; ++m) {
#pragma unroll
                for (int md = 0; md < 3; ++md) {
                    const int lo = (md == 0) ? m + P * ti[1] + P2 * ti[2] : (md == 1) ? ti[0] + P * m + P2 * ti[2] : ti[0] + P * ti[1] + P2 * m;
                    const T dvl = opD<T>(ops, ti[md] * P + m);
#pragma unroll
                    for (int v = 0; v < 5; ++v) hd[v] += dvl * Acc[(md * 5 + v) * P3 + lo];
                }
            }
            const T ci[5] = {Cc[node], Cc[P3 + node], Cc[2 * P3 + node], Cc[3 * P3 + node], Cc[4 * P3 + node]};
            T av[9];
#pragma unroll
            for (int m = 0; m < 9; ++m) av[m] = Av[m * P3 + node];
#pragma unroll
            for (int sd = 0; sd < 3; ++sd) {
#pragma unroll
                for (int lr = 0; lr < 2; ++lr) {
                    if (ti[sd] != (lr ? N : 0)) continue;
                    const int f = 2 * sd + lr;
                    const int q = (sd == 0) ? ti[1] + P * ti[2] : (sd == 1) ? ti[0] + P * ti[2] : ti[0] + P * ti[1];
                    T dn[3] = {J[(sd * 3) * P3 + node], J[(sd * 3 + 1) * P3 + node], J[(sd * 3 + 2) * P3 + node]};
                    T nn = dn[0] * dn[0];
                    nn += dn[1] * dn[1];
                    nn += dn[2] * dn[2];
                    nn = dsqrt(nn);
#pragma unroll
                    for (int d = 0; d < 3; ++d) dn[d] = fdiv(dn[d], nn);
                    T fin[5];
                    dif_flux(ci, av, dn, fin);
                    const T ss = lr ? T(-1) : T(1);
                    const T wend = opW<T>(ops, lr * N);
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        const T fs = -ss * as_real<T>(dv.sf3)[v * dv.nslot + (cell * 6 + f) * P2 + q];
                        hd[v] += fdiv(-ss * (fs - fin[v]) * nn, wend);
                    }
                }
            }
            if (!u64) {
                const T js = fdiv(T(1), T(1) * detJt);
#pragma unroll
                for (int v = 0; v < 5; ++v) hd[v] *= js;
            }
        }
    }

    // ---- phase C: first-order subcell residual, only where alpha > 0
    T lo[5] = {0, 0, 0, 0, 0};
    bool any_lo = false;
#pragma unroll
    for (int k = 0; k < CPB; ++k) {
        const int64_t ck = (int64_t)blockIdx.x * CPB + k;
        if (ck < dv.nc && stored_gt0<T>(dv.alpha[ck])) any_lo = true;
    }
    if (any_lo) {
        __syncthreads();
        const bool do_lo = valid && stored_gt0<T>(alpha);
        if (do_lo) {
            const T fb = (alpha_t <= T(0)) ? T(0) : (alpha_t <= T(1) ? alpha_t : T(1));
            for (int task = node; task < 3 * P2; task += P3) {
                const int dir = task / P2, line = task - dir * P2, la = line % P, lb = line / P;
                T acc[P][5];
#pragma unroll
                for (int i = 0; i < P; ++i)
#pragma unroll
                    for (int v = 0; v < 5; ++v) acc[i][v] = T(0);
                // running subcell normal n_(i-1,i) = Ja_0 + sum_{l<i} sum_m Q_lm Ja_m
                // (metric_terms.cc:106-141)
                const int n0 = line_node<P>(dir, la, lb, 0);
                T sn[3] = {J[(dir * 3) * P3 + n0], J[(dir * 3 + 1) * P3 + n0], J[(dir * 3 + 2) * P3 + n0]};
#pragma unroll
                for (int id = 1; id < P; ++id) {
#pragma unroll
                    for (int m = 0; m < P; ++m) {
                        const int nm = line_node<P>(dir, la, lb, m);
                        const T qlm = opQ<T>(ops, (id - 1) * P + m);
#pragma unroll
                        for (int d = 0; d < 3; ++d) sn[d] += qlm * J[(dir * 3 + d) * P3 + nm];
                    }
                    const int nl = line_node<P>(dir, la, lb, id - 1), nr = line_node<P>(dir, la, lb, id);
                    T nn = sn[0] * sn[0];
                    nn += sn[1] * sn[1];
                    nn += sn[2] * sn[2];
                    nn = dsqrt(nn);
                    const T dn[3] = {fdiv(sn[0], nn), fdiv(sn[1], nn), fdiv(sn[2], nn)};
                    const T cL[5] = {Cc[nl], Cc[P3 + nl], Cc[2 * P3 + nl], Cc[3 * P3 + nl], Cc[4 * P3 + nl]};
                    const T cR[5] = {Cc[nr], Cc[P3 + nr], Cc[2 * P3 + nr], Cc[3 * P3 + nr], Cc[4 * P3 + nr]};
                    T F[5];
                    if constexpr (sizeof(T) == 4) inv_surf_flux_mx(cL, cR, dn, gm, g.isf, fb, F);
                    else inv_surf_flux(cL, cR, dn, gm, g.isf, fb, F);
                    const T wl = opW<T>(ops, id - 1), wr = opW<T>(ops, id);
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        acc[id - 1][v] += fdiv(F[v] * nn, wl);
                        acc[id][v] -= fdiv(F[v] * nn, wr);
                    }
                }
                // cell-face terms at both ends of the line
#pragma unroll
                for (int lr = 0; lr < 2; ++lr) {
                    const int i = lr ? N : 0;
                    const int ni = line_node<P>(dir, la, lb, i);
                    const int f = 2 * dir + lr;
                    const int q = (dir == 0) ? la + P * lb : (dir == 1) ? la + P * lb : la + P * lb;
                    T nn = J[(dir * 3) * P3 + ni] * J[(dir * 3) * P3 + ni];
                    nn += J[(dir * 3 + 1) * P3 + ni] * J[(dir * 3 + 1) * P3 + ni];
                    nn += J[(dir * 3 + 2) * P3 + ni] * J[(dir * 3 + 2) * P3 + ni];
                    nn = dsqrt(nn);
                    const T sg = lr ? T(1) : T(-1);  // contrib_sign and flux_sign
                    const T wend = opW<T>(ops, lr * N);
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        const T fl = sg * as_real<T>(dv.sf)[v * dv.nslot + (cell * 6 + f) * P2 + q];
                        acc[i][v] += fdiv(sg * fl * nn, wend);
                    }
                }
#pragma unroll
                for (int i = 0; i < P; ++i) {
                    const int ni = line_node<P>(dir, la, lb, i);
#pragma unroll
                    for (int v = 0; v < 5; ++v) Acc[(dir * 5 + v) * P3 + ni] = acc[i][v];
                }
            }
        }
        __syncthreads();
        if (do_lo) {
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                const T sum = Acc[v * P3 + node] + Acc[(5 + v) * P3 + node] + Acc[(10 + v) * P3 + node];
                lo[v] = u64 ? sum : fdiv(sum, -detJt);
            }
        }
    }
    if (!valid) return;

    // ---- phase D: blend, then either store the residual or advance the RK registers
    if constexpr (sizeof(T) == 4) {
        if (u64) {
            // MIXED form: the blend of the unscaled FP32 sums, R = (-1/detJ) (alpha lo + (1 - alpha)
            // ho - (1 - alpha_d) hd), scaled in FP64; dt*R, the registers and their combination
            // (update_rk4, dgsem/plens.cc:4353-4400) in FP64
            const double nij = -dv.invJ[dof];
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
#pragma unroll
                for (int v = 0; v < 5; ++v) sa.Rout[v * dv.nd + dof] = Ru[v] * nij;
                return;
            }
            const double sc = nij * rhs_step(dv, cell);  // -dt/detJ
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                const double Rs = Ru[v] * sc;
                const int64_t k = v * dv.nd + dof;
                const double u = dv.U[k];
                double un;
                if (sa.mode == 1) {
                    // U + c0 R0 + c1 R1 + c2 Rs, the chain of the TMA-staged kernel
                    un = u;
                    if (sa.stage >= 3) un = __fma_rn(sa.c0, sa.R0[k], un);
                    if (sa.stage >= 2) un = __fma_rn(sa.c1, sa.R1[k], un);
                    un = __fma_rn(sa.c2, Rs, un);
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
        // MIXED_R32 form: blend and register combination in FP32 (the residual is an FP32
        // result, and so is dt*R, which the registers hold in FP32), the state accumulated in FP64
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
        for (int v = 0; v < 5; ++v) ud[v] = dv.U[v * dv.nd + dof];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const float Rs = R[v] * dtu;
            const int64_t k = v * dv.nd + dof;
            if (sa.mode == 1) {
                float inc;
                if (sa.stage == 1) inc = sa.fc2 * Rs;
                else if (sa.stage == 2) inc = sa.fc1 * as_real<float>(sa.R1)[k] + sa.fc2 * Rs;
                else inc = sa.fc0 * as_real<float>(sa.R0)[k] + sa.fc1 * as_real<float>(sa.R1)[k] + sa.fc2 * Rs;
                if (sa.keep) as_real<float>(sa.Rw)[k] = Rs;
                const double un = ud[v] + f32_to_f64(inc);
                dv.U[k] = un;
                dv.Uf[k] = f64_to_f32(un);
            } else {
                const double Rsd = f32_to_f64(Rs);
                double un;
                if (sa.stage == 1) un = ud[v] + Rsd;
                else if (sa.stage == 2) un = 0.75 * dv.U0[k] + 0.25 * ud[v] + 0.25 * Rsd;
                else un = 1.0 / 3 * dv.U0[k] + 2.0 / 3 * ud[v] + 2.0 / 3 * Rsd;
                dv.U[k] = un;
                dv.Uf[k] = f64_to_f32(un);
            }
        }
        return;
    }
    double R[5];
    const double ad = VISC ? dv.alpha_d[cell] : 0.0;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        if (VISC) R[v] = (1 - ad) * (double)hd[v] + alpha * (double)lo[v] + (1 - alpha) * (double)ho[v];
        else R[v] = alpha * (double)lo[v] + (1 - alpha) * (double)ho[v];
    }
    if (g.plens_2d) R[3] = 0;
    if (sa.mode == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) sa.Rout[v * dv.nd + dof] = R[v];
        return;
    }
    const double dtu = rhs_step(dv, cell);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        const double Rs = R[v] * dtu;
        const int64_t k = v * dv.nd + dof;
        double un;
        if (sa.mode == 1) {
            if (sa.stage == 1) un = ud[v] + sa.c2 * Rs;
            else if (sa.stage == 2) un = ud[v] + (sa.c1 * sa.R1[k] + sa.c2 * Rs);
            else un = ud[v] + (sa.c0 * sa.R0[k] + sa.c1 * sa.R1[k] + sa.c2 * Rs);
            if (sa.keep) sa.Rw[k] = Rs;
        } else {
            if (sa.stage == 1) un = ud[v] + Rs;
            else if (sa.stage == 2) un = 0.75 * dv.U0[k] + 0.25 * ud[v] + 0.25 * Rs;
            else un = 1.0 / 3 * dv.U0[k] + 2.0 / 3 * ud[v] + 2.0 / 3 * Rs;
        }
        dv.U[k] = un;
    }
}

}  // namespace plens_gpu
