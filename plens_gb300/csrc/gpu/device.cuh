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
    float ftv[kMaxP];
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
    double time0;              // clock and step count at the start of the last step (learned
    long long n_steps0;        // sensor: a step that fails the positivity check is redone)
};

struct Dev {
    int64_t nc, nd, ntask, nslot;
    // mesh
    const double *detJ, *Ja, *Jinv, *h_min, *center;
    // the FP32 rounding (f64_to_f32) of detJ, Ja and Jinv, made once on the device at context
    // creation -- the value every FP32 consumer of the FP64 metric terms would compute -- in both
    // mixed forms, none in the FP64 form; where one is null its FP32 consumers round the FP64
    // array themselves
    const float *detJf, *Jaf, *Jinvf;
    // MIXED form: 1/detJ in FP64 (made once at creation), by which the volume kernels scale the
    // FP32 residual sums in FP64 (null otherwise)
    const double* invJ;
    const int32_t *cell_nbr;
    const uint8_t *cell_wall;
    const int32_t *ft_cell, *ft_face, *ft_nbr_cell, *ft_nbr_face, *ft_bc, *ft_nbr_fdof;
    const double *ft_normal, *ft_xyz;
    // per face dof of a face task: the owner-side dof, the neighbour-side dof (interior faces
    // and periodic partners; -1 otherwise), the owner's face slot and the neighbour's face slot
    // (interior faces; -1 otherwise)
    const int32_t *fd_own, *fd_nbr, *fs_own, *fs_nbr;
    // the mixed form's inviscid face list: the face dofs above with each periodic pair of face
    // tasks computed once (the partner's slot receives -F, as an interior face's neighbour does)
    // when the scheme does not read alpha. Per entry two 16-byte words: (own dof, other dof,
    // own slot, other slot) and (the FP32 unit normal, the task face dof as integer bits). The
    // other dof is -1 exactly where a boundary condition supplies the ghost state; the other
    // slot is set for interior faces and merged periodic pairs.
    int64_t n_mx;
    const int4* mx_dofs;
    const float4* mx_geom;
    const plens_bc_desc* bcs;
    int n_bc;
    const plens_expr_insn* expr_code;
    const int32_t *expr_off, *expr_len;
    int n_expr;
    // state
    double* U;
    double* U0;
    float* Uf;  // mixed form: FP32 image of U (round to nearest), kept current by the update
    double *alpha_raw, *alpha, *alpha_d;
    double* tvstat;    // [3][nc] filter statistics of the modal indicator
    double *sf, *sf3;  // surface terms [5][nslot]
    double* avars;     // [9][nd]
    // compacted troubled-cell list of the mixed forms (ordered by cell index): lo_list[pos] =
    // cell, *lo_count cells; lo_blk: troubled cells per 128-cell smoothing block, lo_mask: their
    // warp ballots ([block][4]); lo_decode: 1 when the subcell kernel finds the cell at each list
    // position from lo_blk and lo_mask itself (and writes lo_list), 0 when k_lo_list builds the
    // list first (meshes whose block counts do not fit the subcell kernel's shared memory);
    // lo_buf [5][nd]: the subcell residual sums of each troubled cell at its own dofs
    int32_t* lo_list;
    int32_t* lo_count;
    int32_t* lo_blk;
    uint32_t* lo_mask;
    int lo_decode;
    float* lo_buf;
    // local time stepping (null unless requested): per-cell stable step, and what multiplies
    // each cell's RHS (loc_time_steps)
    double *dt_cell, *dt_loc;
    Scalars* sc;
};

// the factor of a cell's RHS: its local step, or the unclipped global step
__device__ __forceinline__ double rhs_step(const Dev& dv, int64_t cell)
{
    return dv.dt_loc ? dv.dt_loc[cell] : dv.sc->dt_update;
}

__device__ __forceinline__ double eval_expr(const Dev& dv, int idx, double x, double y, double z, double t)
{
    if (idx < 0 || idx >= dv.n_expr) return 0.0 / 0.0;
    const plens_expr_insn* code = dv.expr_code + dv.expr_off[idx];
    const int len = dv.expr_len[idx];
    if (len == 1 && code[0].op == plens::EOP_CONST) return code[0].val;  // a constant: no VM stack
    return plens::expr_eval(code, len, x, y, z, t);
}

// FP64 <-> FP32 conversions by integer arithmetic on the IEEE-754 encodings, with the results of
// the hardware conversions (round to nearest, ties to even). GB300 runs FP64 instructions,
// conversions included, at a small fraction of the FP32 and integer rates, and the mixed form
// converts every FP64 state, metric and register value it reads; these keep that work on the
// integer pipes. Zero and every value whose result is a normal float take the integer path;
// subnormal results, infinities and NaNs (never met on a valid state) use the hardware
// conversion.
__device__ __forceinline__ float f64_to_f32(double x)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned int hi = static_cast<unsigned int>(b >> 32);
    const unsigned int ah = hi & 0x7fffffffu;
    const unsigned int sgn = hi ^ ah;
    // biased FP64 exponent in [897, 1150]: the result is a normal float (or rounds up to inf)
    if (ah - 0x38100000u < 0x0fe00000u) {
        unsigned long long a = b & 0x7fffffffffffffffULL;
        a += 0x0fffffffULL + ((a >> 29) & 1ULL);  // round the 29 dropped bits to nearest even
        return __uint_as_float(sgn | static_cast<unsigned int>((a >> 29) - (896ULL << 23)));
    }
    if (ah < 0x36900000u) return __uint_as_float(sgn);  // |x| < 2^-150 (zero included): rounds to 0
    return __double2float_rn(x);
}

__device__ __forceinline__ double f32_to_f64(float x)
{
    const unsigned int u = __float_as_uint(x);
    const unsigned int au = u & 0x7fffffffu;
    const unsigned int sgn = u ^ au;
    if (au - 0x00800000u < 0x7f000000u)  // normal
        return __hiloint2double(static_cast<int>(sgn | ((au >> 3) + (896u << 20))), static_cast<int>(au << 29));
    if (au == 0) return __hiloint2double(static_cast<int>(sgn), 0);
    return static_cast<double>(x);
}

// a stored FP64 value in the arithmetic type T, and back
template <class T> __device__ __forceinline__ T to_real(double x)
{
    if constexpr (sizeof(T) == 8) return x; else return f64_to_f32(x);
}
template <class T> __device__ __forceinline__ double to_f64(T x)
{
    if constexpr (sizeof(T) == 8) return x; else return f32_to_f64(x);
}

// A metric term in the arithmetic type: the FP64 array (plain form), or its FP32 rounding --
// read from the FP32 image where one exists (MIXED_R32), else rounded from the FP64 array on the
// integer pipes (MIXED); the two are equal bit for bit.
template <class T>
__device__ __forceinline__ T metric(const double* f64, const float* f32, int64_t i)
{
    if constexpr (sizeof(T) == 8) return f64[i];
    else return f32 ? f32[i] : f64_to_f32(f64[i]);
}

// One node's state in the arithmetic type: the FP64 state (plain form) or its FP32 image (mixed).
template <class T>
__device__ __forceinline__ void load_state(const Dev& dv, int64_t dof, T c[5])
{
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        if constexpr (sizeof(T) == 8) c[v] = dv.U[v * dv.nd + dof];
        else c[v] = dv.Uf[v * dv.nd + dof];
    }
}

// The face-value and auxiliary-variable buffers are intermediates of one RHS: the mixed forms
// store them in FP32 inside the FP64-sized allocations. The MIXED_R32 form stores its RK4
// registers (dt*R, an FP32 result there) in FP32 the same way; the MIXED form keeps them in FP64.
template <class T> __device__ __forceinline__ T* as_real(double* p) { return reinterpret_cast<T*>(p); }
template <class T> __device__ __forceinline__ const T* as_real(const double* p) { return reinterpret_cast<const T*>(p); }

// assert_positivity (dgsem/plens.cc:2531-2546, navier_stokes.cc:326-337): rho > 0 and e > 0,
// decided in FP64 with the reference's expressions.
__device__ __forceinline__ bool positive_state_f64(const double c[5])
{
    if (!(c[0] > 0)) return false;
    double ske = c[1] * c[1];
    ske += c[2] * c[2];
    ske += c[3] * c[3];
    const double ri = 1.0 / c[0];
    ske *= 0.5 * ri;
    return (c[4] - ske) * ri > 0;
}

// The same decision for the mixed form: an FP32 screen on 2 rho (rho E) - |rho u|^2, whose
// rounding error is below 1e-6 of the sum of the magnitudes of its terms, accepts the state
// when it clears that sum by 1e-5; any other state is decided by the FP64 test above.
__device__ __forceinline__ bool positive_screen_f32(const float cf[5])
{
    const float a = 2.0f * cf[0] * cf[4];
    float m = cf[1] * cf[1];
    m += cf[2] * cf[2];
    m += cf[3] * cf[3];
    return cf[0] > 0.0f && cf[4] > 0.0f && a - m > 1e-5f * (a + m);
}
__device__ __forceinline__ bool positive_state_screened(const double c[5], const float cf[5])
{
    return positive_screen_f32(cf) || positive_state_f64(c);
}
// the screen on the FP32 image; the FP64 state is read only when the screen does not decide
__device__ __forceinline__ bool positive_dof_screened(const Dev& dv, int64_t dof, const float cf[5])
{
    if (positive_screen_f32(cf)) return true;
    double c[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) c[v] = dv.U[v * dv.nd + dof];
    return positive_state_f64(c);
}

// x > 0 for a stored FP64 value: compared in FP64 by the plain form, on the encoding by the
// mixed form (sign clear and not zero)
template <class T> __device__ __forceinline__ bool stored_gt0(double x)
{
    if constexpr (sizeof(T) == 8) return x > 0; else return __double_as_longlong(x) > 0;
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

// Node order of the thread-written per-node shared arrays of the line-task kernels (the mixed
// volume and subcell kernels) at P = 4: node n = x + 4 y + 16 z is stored at (x ^ z) +
// 4 (y ^ x) + 16 z (the identity at other degrees), with the two cells of a block 16 banks apart.
// Their line phases give each warp one direction, its lanes the 16 lines of both cells: at every
// position along the lines the 32 lanes then read 32 different banks in all three directions,
// and 32 consecutive nodes of one cell (the per-node phases) do too. In the plain order the x
// and y lines put two lanes on each bank.
template <int P>
__device__ __forceinline__ int swz(int n)
{
    if constexpr (P == 4) {
        const int x = n & 3, y = (n >> 2) & 3, z = n >> 4;
        return (x ^ z) | ((y ^ x) << 2) | (z << 4);
    } else {
        return n;
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
