// launch.cuh -- host-side launchers of the templated kernels, gathered into a table per
// (P, arithmetic type) so the context can dispatch on the run-time degree and precision.
#pragma once

#include "blender_tc.cuh"
#include "kernels.cuh"
#include "subcell_mx.cuh"
#include "surface_mx.cuh"
#include "volume_mx.cuh"

namespace plens_gpu {

struct LaunchTable {
    int P = 0;
    // each returns the number of kernels it launched
    int (*blender)(const Dev&, const Ops&, const GasP&, const BlendP&, cudaStream_t) = nullptr;
    // the mixed forms' modal indicator with the change of basis on the tensor cores (N = 3 only;
    // blender_tc.cuh), given its B operand
    int (*blender_tc)(const Dev&, const Ops&, const GasP&, const BlendP&, const float*, cudaStream_t) = nullptr;
    int (*surface)(int stage, const Dev&, const GasP&, double* out, cudaStream_t) = nullptr;
    int (*aux)(const Dev&, const Ops&, const GasP&, cudaStream_t) = nullptr;
    int (*volume)(bool visc, const Dev&, const Ops&, const GasP&, const StageArgs&, cudaStream_t) = nullptr;
    int (*time_step)(const Dev&, const GasP&, double N15, int N, cudaStream_t) = nullptr;
    // the subcell residual over the compacted troubled-cell list, where the volume kernel takes it
    // from there (the TMA-staged mixed kernel); 0 launches otherwise
    bool (*uses_lo_list)(const GasP&) = nullptr;
    int (*subcell)(const Dev&, const Ops&, const GasP&, cudaStream_t) = nullptr;
};

LaunchTable table_fp64(int P);
LaunchTable table_mixed(int P);

template <int P, class T>
struct Launch {
    using CB = CellBlock<P>;
    static int grid_cells(int64_t nc) { return (int)((nc + CB::CPB - 1) / CB::CPB); }

    static int blender(const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, cudaStream_t st)
    {
        k_blender<P, T><<<grid_cells(dv.nc), CB::THREADS, 0, st>>>(dv, ops, g, bp);
        return 1;
    }
    static int blender_tc(const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, const float* Btc, cudaStream_t st)
    {
        static int nsm = 0;
        if (!nsm) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaFuncSetAttribute(k_blender_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BtcSmem::bytes);
            if (nsm < 1) nsm = 1;
        }
        const int tr = tc::tile_rows(dv.nc, nsm);
        const int64_t tiles = (dv.nc + tr - 1) / tr;
        k_blender_tc<P><<<(unsigned)(tiles < nsm ? tiles : nsm), kBtcThreads, BtcSmem::bytes, st>>>(dv, Btc, g, bp, ops, tr);
        return 1;
    }
    template <bool HLLC>
    static void surface_inv_mx(const Dev& dv, const GasP& g, double* out, cudaStream_t st)
    {
        static int blocks = 0;
        if (!blocks) {
            int dev = 0, nsm = 0, occ = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_surface_inv_mx<P, HLLC>, 128, 0);
            blocks = (occ > 0 ? occ : 1) * (nsm > 0 ? nsm : 1);
        }
        const int64_t need = (dv.n_mx + 127) / 128;
        k_surface_inv_mx<P, HLLC><<<(int)(need < blocks ? need : blocks), 128, 0, st>>>(dv, g, out);
    }
    static int surface(int stage, const Dev& dv, const GasP& g, double* out, cudaStream_t st)
    {
        const int64_t n = dv.ntask * P * P;
        const int grid = (int)((n + 127) / 128);
        if constexpr (sizeof(T) == 4) {
            if (stage == 2) {  // persistent, software-pipelined
                if (g.isf == PLENS_ISF_HLLC) surface_inv_mx<true>(dv, g, out, st);
                else surface_inv_mx<false>(dv, g, out, st);
                return 1;
            }
        }
        if (stage == 1) k_surface<P, T, 1><<<grid, 128, 0, st>>>(dv, g, out);
        else if (stage == 2) k_surface<P, T, 2><<<grid, 128, 0, st>>>(dv, g, out);
        else k_surface<P, T, 3><<<grid, 128, 0, st>>>(dv, g, out);
        return 1;
    }
    static int aux(const Dev& dv, const Ops& ops, const GasP& g, cudaStream_t st)
    {
        const size_t bytes = sizeof(T) * (size_t)CB::CPB * (5 * CB::P3 + 9 * CB::P3 + 30 * CB::P2);
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_aux<P, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            attr = true;
        }
        k_aux<P, T><<<grid_cells(dv.nc), CB::THREADS, bytes, st>>>(dv, ops, g);
        return 1;
    }
    template <bool VISC, bool R64>
    static void volume_mx(const Dev& dv, const Ops& ops, const GasP& g, const StageArgs& sa, cudaStream_t st)
    {
        if constexpr (P % 2 == 0) {
            const size_t bytes = MxSmem<P, VISC, R64>::bytes;
            static bool attr = false;
            if (!attr) {
                cudaFuncSetAttribute(k_volume_mx<P, VISC, R64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
                attr = true;
            }
            k_volume_mx<P, VISC, R64><<<grid_cells(dv.nc), CB::THREADS, bytes, st>>>(dv, ops, g, sa);
        }
    }
    static int volume(bool visc, const Dev& dv, const Ops& ops, const GasP& g, const StageArgs& sa, cudaStream_t st)
    {
        // mixed form, even P, Chandrashekhar volume flux (the configurations' scheme): the
        // TMA-staged kernel; the other volume fluxes take the generic kernel
        if constexpr (sizeof(T) == 4 && P % 2 == 0) {
            if (g.ivf == PLENS_IVF_CHANDRASHEKHAR) {
                if (sa.reg64) {
                    if (visc) volume_mx<true, true>(dv, ops, g, sa, st);
                    else volume_mx<false, true>(dv, ops, g, sa, st);
                } else {
                    if (visc) volume_mx<true, false>(dv, ops, g, sa, st);
                    else volume_mx<false, false>(dv, ops, g, sa, st);
                }
                return 1;
            }
        }
        const size_t bytes = VolSmem<P, T>::bytes(visc);
        if (visc) {
            static bool attr = false;
            if (!attr) {
                cudaFuncSetAttribute(k_volume<P, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
                attr = true;
            }
            k_volume<P, T, true><<<grid_cells(dv.nc), CB::THREADS, bytes, st>>>(dv, ops, g, sa);
        } else {
            static bool attr = false;
            if (!attr) {
                cudaFuncSetAttribute(k_volume<P, T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
                attr = true;
            }
            k_volume<P, T, false><<<grid_cells(dv.nc), CB::THREADS, bytes, st>>>(dv, ops, g, sa);
        }
        return 1;
    }
    static bool uses_lo_list(const GasP& g)
    {
        return sizeof(T) == 4 && P % 2 == 0 && g.ivf == PLENS_IVF_CHANDRASHEKHAR;
    }
    template <bool HLLC>
    static void subcell_launch(const Dev& dv, const Ops& ops, const GasP& g, cudaStream_t st)
    {
        // persistent grid, at most four blocks per SM: the blocks take the listed cells in groups
        // (against two per SM: shock-vortex 64^3 18.75 -> 18.49 ms per step, the DMR and the
        // cylinder unchanged, A/B on the same box)
        static int blocks = 0;
        if (!blocks) {
            int dev = 0, nsm = 0, occ = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_subcell_lo<P, HLLC>, CB::THREADS, 0);
            blocks = (occ > 4 ? 4 : (occ > 0 ? occ : 1)) * (nsm > 0 ? nsm : 1);
        }
        const int64_t need = (dv.nc + CB::CPB - 1) / CB::CPB;
        // decoding: the prefix sums of the smoothing blocks' counts in dynamic shared memory
        const int bytes = dv.lo_decode ? (int)(4 * ((dv.nc + kSmoothThreads - 1) / kSmoothThreads + 1)) : 0;
        static int attr = 0;
        if (bytes > attr) {
            cudaFuncSetAttribute(k_subcell_lo<P, HLLC>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            attr = bytes;
        }
        k_subcell_lo<P, HLLC><<<(int)(need < blocks ? need : blocks), CB::THREADS, bytes, st>>>(dv, ops, g);
    }
    static int subcell(const Dev& dv, const Ops& ops, const GasP& g, cudaStream_t st)
    {
        if (!uses_lo_list(g)) return 0;
        if (g.isf == PLENS_ISF_HLLC) subcell_launch<true>(dv, ops, g, st);
        else subcell_launch<false>(dv, ops, g, st);
        return 1;
    }
    static int time_step(const Dev& dv, const GasP& g, double N15, int N, cudaStream_t st)
    {
        if (dv.dt_cell) {  // local stepping: per-cell steps as well
            k_time_step_cells<P, T><<<(unsigned)((dv.nc + 7) / 8), 256, 0, st>>>(dv, g, N15, N);
            return 1;
        }
        const int64_t per_block = 256 * kStepItems<T>;
        const int grid = (int)((dv.nd + per_block - 1) / per_block);
        k_time_step<P, T><<<grid, 256, 0, st>>>(dv, g, N15, N);
        return 1;
    }
    static LaunchTable table()
    {
        LaunchTable t;
        t.P = P;
        t.blender = &blender;
        if constexpr (sizeof(T) == 4 && P == 4) t.blender_tc = &blender_tc;
        t.surface = &surface;
        t.aux = &aux;
        t.volume = &volume;
        t.time_step = &time_step;
        t.uses_lo_list = &uses_lo_list;
        t.subcell = &subcell;
        return t;
    }
};

}  // namespace plens_gpu
