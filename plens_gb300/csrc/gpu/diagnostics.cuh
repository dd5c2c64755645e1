// diagnostics.cuh -- the error norms that PLENS::write logs at output steps (dgsem/plens.cc:
// 4234-4243): the steady-state error of calc_ss_error (3985-4035) and the density error of
// calc_convergence_error (4044-4098). Both are L2 norms by QGauss(N+1) quadrature of the DG field
// (VectorTools::integrate_difference), i.e. sqrt(sum over cells and Gauss points of w |J| f^2),
// with f interpolated from the GLL nodes to the Gauss points by sum factorisation.
#pragma once

#include "kernels.cuh"

namespace plens_gpu {

// 1D interpolation GLL nodes -> Gauss points: g[q * P + i] = l_i(xi_q)
struct GaussInterp {
    double g[kMaxP * kMaxP];
};

// rho E at the start of the step (PLENS::rhoE_old is set from g_cvars at the end of update(),
// dgsem/plens.cc:4507, i.e. it holds the previous step's starting rho E)
static __global__ void k_save_rhoE(Dev dv, double* rhoE_old)
{
    if (!dv.sc->active) return;
    const double* E = dv.U + 4 * dv.nd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dv.nd; i += (int64_t)gridDim.x * blockDim.x)
        rhoE_old[i] = E[i];
}

// One block per cell, one thread per Gauss point. Per cell: the quadrature sums of rho E^2, of
// ((rho E - rho E_old) / loc_dt)^2 and of (rho - exact)^2 (the last only with an expression).
template <int P>
__global__ void __launch_bounds__(((P * P * P + 31) / 32) * 32) k_cell_errors(
    Dev dv, GaussInterp gi, const double* __restrict__ rhoE_old, const double* __restrict__ q_wJ,
    const double* __restrict__ q_xyz, int expr_exact, double* __restrict__ cell_sums)
{
    constexpr int P2 = P * P, P3 = P2 * P, NW = (P3 + 31) / 32;
    __shared__ double a[3][P3], b[3][P3];
    __shared__ double red[3][NW];
    const int64_t c = blockIdx.x;
    const int t = threadIdx.x;
    const bool conv = expr_exact >= 0;
    const double dt = rhs_step(dv, c);
    if (t < P3) {
        const int64_t dof = c * P3 + t;
        const double E = dv.U[4 * dv.nd + dof];
        a[0][t] = E;
        a[1][t] = rhoE_old ? (E - rhoE_old[dof]) / dt : 0.0;
        a[2][t] = dv.U[dof];
    }
    __syncthreads();
    // x, then y, then z: b <- along x of a; a <- along y of b; b <- along z of a
    const int i = t % P, j = (t / P) % P, k = t / P2;
    if (t < P3)
        for (int f = 0; f < 3; ++f) {
            double s = 0;
            for (int m = 0; m < P; ++m) s += gi.g[i * P + m] * a[f][m + P * j + P2 * k];
            b[f][t] = s;
        }
    __syncthreads();
    if (t < P3)
        for (int f = 0; f < 3; ++f) {
            double s = 0;
            for (int m = 0; m < P; ++m) s += gi.g[j * P + m] * b[f][i + P * m + P2 * k];
            a[f][t] = s;
        }
    __syncthreads();
    double v[3] = {0, 0, 0};
    if (t < P3) {
        const int64_t q = c * P3 + t;
        double u[3];
        for (int f = 0; f < 3; ++f) {
            double s = 0;
            for (int m = 0; m < P; ++m) s += gi.g[k * P + m] * a[f][i + P * j + P2 * m];
            u[f] = s;
        }
        if (conv)
            u[2] -= eval_expr(dv, expr_exact, q_xyz[q], q_xyz[dv.nd + q], q_xyz[2 * dv.nd + q], dv.sc->time);
        const double w = q_wJ[q];
        for (int f = 0; f < 3; ++f) v[f] = w * u[f] * u[f];
    }
    for (int f = 0; f < 3; ++f) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[f] += __shfl_down_sync(0xffffffffu, v[f], off);
        if ((t & 31) == 0) red[f][t >> 5] = v[f];
    }
    __syncthreads();
    if (t < 3) {
        double s = 0;
        for (int w = 0; w < NW; ++w) s += red[t][w];
        cell_sums[t * dv.nc + c] = (t == 2 && !conv) ? 0.0 : s;
    }
}

// the three domain sums, in a fixed order (one block)
static __global__ void __launch_bounds__(1024) k_sum_errors(const double* __restrict__ cell_sums, int64_t nc,
                                                            double* __restrict__ out)
{
    __shared__ double red[32];
    for (int f = 0; f < 3; ++f) {
        double s = 0;
        for (int64_t c = threadIdx.x; c < nc; c += blockDim.x) s += cell_sums[f * nc + c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
            out[f] = tot;
        }
        __syncthreads();
    }
}

}  // namespace plens_gpu
