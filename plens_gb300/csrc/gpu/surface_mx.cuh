// surface_mx.cuh -- the mixed form's inviscid face-flux kernel (calc_surf_flux stage 2,
// dgsem/plens.cc:1717-1913): the work of k_surface<P, float, 2> as a persistent, software-
// pipelined loop. The kernel is bound by the latency of its gathers: a face dof's two states are
// found through the precomputed dof tables (a dependent load), so each thread keeps two face dofs
// in flight -- the tables of the face dof after next and the states of the next one are loading
// while it evaluates the current one.
#pragma once

#include "kernels.cuh"

namespace plens_gpu {

// per face dof: what the loop carries between iterations
struct FaceItem {
    int32_t idx;      // face dof of the task list (-1: none)
    int32_t gd, gdn;  // own dof, other dof (interior or periodic partner; -1 where a BC gives the ghost)
    int32_t slot, slot_nb;  // face slots of both sides (-1: no neighbour slot)
    float n[3];
};

// entry i of the mixed face list: two 16-byte loads
__device__ __forceinline__ FaceItem face_item(const Dev& dv, int64_t i, int64_t total)
{
    FaceItem it;
    it.idx = -1;
    if (i < total) {
        const int4 a = __ldg(dv.mx_dofs + i);
        const float4 b = __ldg(dv.mx_geom + i);
        it.gd = a.x;
        it.gdn = a.y;
        it.slot = a.z;
        it.slot_nb = a.w;
        it.n[0] = b.x;
        it.n[1] = b.y;
        it.n[2] = b.z;
        it.idx = __float_as_int(b.w);
    }
    return it;
}

__device__ __forceinline__ void face_states(const Dev& dv, const FaceItem& it, float cs[5], float c2[5])
{
    if (it.idx < 0) return;
    load_state<float>(dv, it.gd, cs);
    if (it.gdn >= 0) load_state<float>(dv, it.gdn, c2);
}

// HLLC: the configurations' surface flux, instantiated on its own so that the kernel carries no
// code of the other schemes (the alpha-blended ones read alpha; HLLC does not)
template <int P, bool HLLC>
__global__ void __launch_bounds__(128, HLLC ? 5 : 4) k_surface_inv_mx(Dev dv, GasP g, double* out)
{
    constexpr int P2 = P * P;
    Scalars* s = dv.sc;
    if (!s->active) return;
    const int64_t total = dv.n_mx;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const float gm = f64_to_f32(g.gamma);
    const bool blended = !HLLC && (g.isf == PLENS_ISF_CHANDRASHEKHAR || g.isf == PLENS_ISF_RUSANOV_HLLC ||
                                   g.isf == PLENS_ISF_RUSANOV_AUSM_PLUS_UP);
    float* o = as_real<float>(out);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    FaceItem cur = face_item(dv, i, total);
    FaceItem nxt = face_item(dv, i + stride, total);
    float cs[5], c2[5];
    face_states(dv, cur, cs, c2);
    while (cur.idx >= 0) {
        // in flight during this face dof's flux: the next one's states, the one after's tables
        float ns[5], n2[5];
        face_states(dv, nxt, ns, n2);
        const FaceItem aft = face_item(dv, i + 2 * stride, total);
        i += stride;

        const int64_t ti = cur.idx / P2;
        float fb = 0.0f;
        if (blended) {
            // own alpha on boundary faces (periodic included: not merged for these schemes),
            // the mean of both cells' on interior faces (the only ones with a neighbour slot)
            const int64_t c = dv.ft_cell[ti];
            float a = f64_to_f32(dv.alpha[c]);
            if (cur.slot_nb >= 0) a = 0.5f * (a + f64_to_f32(dv.alpha[dv.ft_nbr_cell[ti]]));
            fb = (a <= 0.0f) ? 0.0f : (a <= 1.0f ? a : 1.0f);
        }
        if (cur.gdn < 0) {  // a boundary condition gives the ghost state (periodic: the partner's)
            const plens_bc_desc& b = dv.bcs[dv.ft_bc[ti]];
            float av[9] = {}, ag[9];
            bc_ghost<float>(2, dv, g, b, cs, av, cur.n, dv.ft_xyz + (int64_t)cur.idx * 3, s->time, -1, c2, ag);
        }
        float fl[5];
        if constexpr (HLLC) hllc_n_f32(cs, c2, cur.n, gm, fl);
        else inv_surf_flux_mx(cs, c2, cur.n, gm, g.isf, fb, fl);
        const int64_t slot = cur.slot, slot_nb = cur.slot_nb;
#pragma unroll
        for (int v = 0; v < 5; ++v) o[v * dv.nslot + slot] = fl[v];
        if (slot_nb >= 0)
#pragma unroll
            for (int v = 0; v < 5; ++v) o[v * dv.nslot + slot_nb] = -fl[v];

        cur = nxt;
        nxt = aft;
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            cs[v] = ns[v];
            c2[v] = n2[v];
        }
    }
}

}  // namespace plens_gpu
