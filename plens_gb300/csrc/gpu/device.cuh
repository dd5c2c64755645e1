// device.cuh -- device-side data view and shared helpers of the hot-path kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../common/expr.h"
#include "plens_gpu.h"

namespace plens_gpu {

constexpr int kMaxP = 6;

// 1D operators on the GLL nodes of [0,1] (dgsem/plens.cc:1646-1663) and the 1D change of basis
// C1[a][i] = int_0^1 psi_a l_i (the tensor factor of dgsem/change_of_basis_matrix.h:74-98).
struct Ops {
    double w[kMaxP];
    double D[kMaxP * kMaxP];
    double Q[kMaxP * kMaxP];
    double C1[kMaxP * kMaxP];
    double tv[kMaxP];  // total variation of the 1D Legendre modes (blender_calculator.cc:69-86)
    // FP32 copies for the mixed form (the operators are consumed in the arithmetic type)
    float fw[kMaxP];
    float fD[kMaxP * kMaxP];
    float fQ[kMaxP * kMaxP];
    float fC1[kMaxP * kMaxP];
};

template <class T> __device__ __forceinline__ T opC1(const Ops& o, int i)
{
    if constexpr (sizeof(T) == 8) return o.C1[i]; else return o.fC1[i];
}

template <class T> __device__ __forceinline__ T opD(const Ops& o, int i)
{
    if constexpr (sizeof(T) == 8) return o.D[i]; else return o.fD[i];
}
// 2*D_ij: scaling by 2 is exact, so (2*D)*norm equals the reference's 2*D*norm bitwise
template <class T> __device__ __forceinline__ T opD2(const Ops& o, int i)
{
    if constexpr (sizeof(T) == 8) return 2.0 * o.D[i]; else return 2.0f * o.fD[i];
}
template <class T> __device__ __forceinline__ T opQ(const Ops& o, int i)
{
    if constexpr (sizeof(T) == 8) return o.Q[i]; else return o.fQ[i];
}
template <class T> __device__ __forceinline__ T opW(const Ops& o, int i)
{
    if constexpr (sizeof(T) == 8) return o.w[i]; else return o.fw[i];
}

struct GasP {
    double gamma, R, Pr, mu0, T0, S;
    int const_visc, inviscid, isf, ivf, plens_2d;
};

struct BlendP {
    double thr, sharp, amin, amax;
    int func;      // 0 Hennemann, 1 linear
    int var;       // 0 pxrho, 1 p, 2 rho
    int expr_wall, expr_vis, expr_courant;
    int do_filter;
    int gate;      // 1: the plain blender runs only while the learned sensor is in fallback
    const uint8_t* mask;  // if set (and not in fallback): the plain blender runs only on cells with mask 1
};

// Device scalars of one context, in one allocation.
struct Scalars {
    double time;        // PLENS::cur_time
    double dt;          // PLENS::time_step after the end-time clip (advances the clock)
    double dt_update;   // PLENS::loc_time_steps (unclipped; multiplies the RHS)
    double end_time;
    double courant;     // Courant number of the current step
    unsigned long long dtmin;  // order-preserving image of the running min of the stable step
    long long n_steps;
    long long bad_dof;
    int active;         // 1 while the current step runs
    int err;            // PLENS_GPU_E_* raised on the device
    long long lo_cells;        // cells the subcell kernel ran on (learned sensor)
    long long judged, fallbacks;
    double max_alpha_err;
    int sensor_fallback;       // 1: this step uses the plain blender
    int pad;
};

struct Dev {
    int64_t nc, nd, ntask, nslot;
    // mesh
    const double *detJ, *Ja, *Jinv, *h_min, *center;
    const int32_t *cell_nbr;
    const uint8_t *cell_wall;
    const int32_t *ft_cell, *ft_face, *ft_nbr_cell, *ft_nbr_face, *ft_bc, *ft_nbr_fdof;
    const double *ft_normal, *ft_xyz;
    const plens_bc_desc* bcs;
    int n_bc;
    const plens_expr_insn* expr_code;
    const int32_t *expr_off, *expr_len;
    int n_expr;
    // state
    double* U;
    double* U0;
    double *alpha_raw, *alpha, *alpha_d;
    double* tvstat;    // [3][nc] filter statistics of the modal indicator
    double *sf, *sf3;  // surface terms [5][nslot]
    double* avars;     // [9][nd]
    int32_t* lo_list;  // compacted troubled-cell list
    int32_t* lo_count;
    Scalars* sc;
};

__device__ __forceinline__ double eval_expr(const Dev& dv, int idx, double x, double y, double z, double t)
{
    if (idx < 0 || idx >= dv.n_expr) return 0.0 / 0.0;
    return plens::expr_eval(dv.expr_code + dv.expr_off[idx], dv.expr_len[idx], x, y, z, t);
}

__device__ __forceinline__ unsigned long long ord_double(double x)
{
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
    return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}
__host__ __device__ inline double unord_double(unsigned long long u)
{
    const unsigned long long b = (u & 0x8000000000000000ULL) ? (u & ~0x8000000000000000ULL) : ~u;
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}
inline unsigned long long ord_double_host(double x)
{
    unsigned long long u;
    memcpy(&u, &x, sizeof(u));
    return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}

// Threads per block and cells per block of the cell-wise kernels: one thread per GLL node,
// several small cells per block.
template <int P>
struct CellBlock {
    static constexpr int P2 = P * P, P3 = P2 * P;
    static constexpr int CPB = (P3 >= 128) ? 1 : 128 / P3;
    static constexpr int THREADS = ((CPB * P3 + 31) / 32) * 32;
};

// face dof -> cell dof (dgsem/face_dof_info.h:92-150)
template <int P>
__device__ __forceinline__ int face_node(int f, int q)
{
    constexpr int P2 = P * P, N = P - 1;
    switch (f) {
    case 0: return P * q;
    case 1: return N + P * q;
    case 2: return (q % P) + P2 * (q / P);
    case 3: return P * N + (q % P) + P2 * (q / P);
    case 4: return q;
    default: return N * P2 + q;
    }
}

// node index of position i along direction dir on the line (a, b) of the other two directions
template <int P>
__device__ __forceinline__ int line_node(int dir, int a, int b, int i)
{
    constexpr int P2 = P * P;
    return (dir == 0) ? i + P * a + P2 * b : (dir == 1) ? a + P * i + P2 * b : a + P * b + P2 * i;
}

}  // namespace plens_gpu
