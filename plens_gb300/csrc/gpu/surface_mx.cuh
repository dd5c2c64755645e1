// surface_mx.cuh -- the mixed form's inviscid face-flux kernel (calc_surf_flux stage 2,
// dgsem/plens.cc:1717-1913): k_surface<P, float, 2> with two face dofs per thread. The kernel is
// bound by the latency of its gathers (the two states of a face dof are found through the
// precomputed dof tables), so each thread first issues the loads of both of its face dofs and
// then evaluates both fluxes.
#pragma once

#include "kernels.cuh"

namespace plens_gpu {

template <int P>
__global__ void __launch_bounds__(128, 6) k_surface_inv_mx(Dev dv, GasP g, double* out)
{
    constexpr int P2 = P * P, K = 2;
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int64_t total = dv.ntask * P2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const float gm = f64_to_f32(g.gamma);
    const bool blended = g.isf == PLENS_ISF_CHANDRASHEKHAR || g.isf == PLENS_ISF_RUSANOV_HLLC ||
                         g.isf == PLENS_ISF_RUSANOV_AUSM_PLUS_UP;
    int64_t idx[K], gd[K], gdn[K];
    int bc[K];
    bool ok[K];
    float cs[K][5], c2[K][5], n[K][3];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        idx[k] = i0 + k * stride;
        ok[k] = idx[k] < total;
        if (ok[k]) {
            bc[k] = dv.ft_bc[idx[k] / P2];
            gd[k] = dv.fd_own[idx[k]];
            gdn[k] = dv.fd_nbr[idx[k]];
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (!ok[k]) continue;
        load_state<float>(dv, gd[k], cs[k]);
        if (gdn[k] >= 0) load_state<float>(dv, gdn[k], c2[k]);
#pragma unroll
        for (int d = 0; d < 3; ++d) n[k][d] = f64_to_f32(dv.ft_normal[idx[k] * 3 + d]);
    }
    float* o = as_real<float>(out);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (!ok[k]) continue;
        const int64_t ti = idx[k] / P2;
        float fb = 0.0f;
        if (blended) {
            const int64_t c = dv.ft_cell[ti];
            float a = f64_to_f32(dv.alpha[c]);
            if (bc[k] < 0) a = 0.5f * (a + f64_to_f32(dv.alpha[dv.ft_nbr_cell[ti]]));
            fb = (a <= 0.0f) ? 0.0f : (a <= 1.0f ? a : 1.0f);
        }
        if (bc[k] >= 0) {
            const plens_bc_desc& b = dv.bcs[bc[k]];
            if (b.type != PLENS_BC_PERIODIC) {  // periodic: the partner's state is the ghost
                float av[9] = {}, ag[9];
                bc_ghost<float>(2, dv, g, b, cs[k], av, n[k], dv.ft_xyz + idx[k] * 3, s->time, -1, c2[k], ag);
            }
        }
        float fl[5];
        inv_surf_flux_mx(cs[k], c2[k], n[k], gm, g.isf, fb, fl);
        const int64_t slot = dv.fs_own[idx[k]], slot_nb = dv.fs_nbr[idx[k]];
#pragma unroll
        for (int v = 0; v < 5; ++v) o[v * dv.nslot + slot] = fl[v];
        if (slot_nb >= 0)
#pragma unroll
            for (int v = 0; v < 5; ++v) o[v * dv.nslot + slot_nb] = -fl[v];
    }
}

}  // namespace plens_gpu
