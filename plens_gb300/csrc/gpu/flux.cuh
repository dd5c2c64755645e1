// flux.cuh -- device restatement of the NavierStokes flux functions
// (modelling/navier_stokes.{h,cc}), templated on the arithmetic type: double for the plain path,
// float for the mixed path. Formulas and branch conditions follow the cited reference lines; the
// per-node quantities (1/rho, velocity, p, beta) are computed once per node with the reference's
// own expressions, so reusing them is bitwise identical to recomputing them per pair.
#pragma once

#include <cuda_runtime.h>

#include "plens_gpu.h"

namespace plens_gpu {

template <class T>
struct GasT {
    T gma, R;
    int isf;
    bool inviscid;
};

template <class T> __device__ __forceinline__ T dsqrt(T x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <class T> __device__ __forceinline__ T dlog(T x) { return log(x); }
template <> __device__ __forceinline__ float dlog<float>(float x) { return logf(x); }
template <class T> __device__ __forceinline__ T dpow(T x, T y) { return pow(x, y); }
// FP32: the base is a positive pressure or speed ratio on every call of this path
template <> __device__ __forceinline__ float dpow<float>(float x, float y) { return __powf(x, y); }
template <class T> __device__ __forceinline__ T dabs(T x) { return fabs(x); }
template <> __device__ __forceinline__ float dabs<float>(float x) { return fabsf(x); }

// Division and logarithm: IEEE division / libm log in FP64 (the plain form reproduces the
// reference's arithmetic); the fast hardware approximations in FP32 (the mixed form, whose
// accuracy target is a relative L1 error of 1e-4).
template <class T> __device__ __forceinline__ T fdiv(T a, T b) { return a / b; }
template <> __device__ __forceinline__ float fdiv<float>(float a, float b) { return __fdividef(a, b); }
template <class T> __device__ __forceinline__ T flog(T x) { return log(x); }
template <> __device__ __forceinline__ float flog<float>(float x) { return __logf(x); }

template <class T>
__device__ __forceinline__ T get_p(const T c[5], T gma)  // navier_stokes.cc:375-383
{
    T ske = c[1] * c[1];
    ske += c[2] * c[2];
    ske += c[3] * c[3];
    ske *= fdiv(T(0.5), c[0]);
    return (gma - 1) * (c[4] - ske);
}

template <class T>
__device__ __forceinline__ T get_e(const T c[5])  // navier_stokes.cc:349-359
{
    T ske = c[1] * c[1];
    ske += c[2] * c[2];
    ske += c[3] * c[3];
    const T ri = T(1) / c[0];
    ske *= T(0.5) * ri;
    return (c[4] - ske) * ri;
}

// logarithmic mean with the series branch for nearly equal arguments (navier_stokes.h:494-501)
template <class T>
__device__ __forceinline__ T log_avg(T xl, T xr)
{
    const T xi = fdiv(xl, xr), f = fdiv(xi - 1, xi + 1), u = f * f;
    T F;
    if constexpr (sizeof(T) == 8) {
        F = (u < T(1e-2)) ? T(1) + u / T(3) + u * u / T(5) + u * u * u / T(7) : T(0.5) * dlog(xi) / f;
    } else {
        F = (u < T(1e-2)) ? T(1) + u * T(1.0 / 3) + u * u * T(0.2) + u * u * u * T(1.0 / 7)
                          : fdiv(T(0.5) * flog(xi), f);
    }
    return fdiv(T(0.5) * (xl + xr), F);
}

// physical inviscid flux along a unit direction (navier_stokes.cc:424-442)
template <class T>
__device__ __forceinline__ void inv_flux(const T c[5], const T dir[3], T gma, T f[5])
{
    const T ri = fdiv(T(1.0), c[0]);
    const T v0 = c[1] * ri, v1 = c[2] * ri, v2 = c[3] * ri;
    const T p = get_p(c, gma);
    T vn = v0 * dir[0];
    vn += v1 * dir[1];
    vn += v2 * dir[2];
    f[0] = c[0] * vn;
    f[1] = vn * c[1] + p * dir[0];
    f[2] = vn * c[2] + p * dir[1];
    f[3] = vn * c[3] + p * dir[2];
    f[4] = (c[4] + p) * vn;
}

// Chandrashekhar two-point volume flux (navier_stokes.cc:1510-1542). q1/q2 hold the per-node
// quantities {rho, 1/rho, v0, v1, v2, p, beta}.
template <class T>
__device__ __forceinline__ void chandrashekhar_vol(const T q1[7], const T q2[7], const T dir[3], T gma, T f[5])
{
    const T beta_ln = log_avg(q1[6], q2[6]);
    const T p_hat = fdiv(T(0.5) * (q1[0] + q2[0]), q1[6] + q2[6]);
    const T rho_ln = log_avg(q1[0], q2[0]);
    T va[3], vsq[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        va[d] = T(0.5) * (q1[2 + d] + q2[2 + d]);
        vsq[d] = T(0.5) * (q1[2 + d] * q1[2 + d] + q2[2 + d] * q2[2 + d]);
    }
    T H = fdiv(T(0.5), (gma - 1) * beta_ln) + fdiv(p_hat, rho_ln);
#pragma unroll
    for (int d = 0; d < 3; ++d) H += va[d] * va[d] - T(0.5) * vsq[d];
    T vn = va[0] * dir[0];
    vn += va[1] * dir[1];
    vn += va[2] * dir[2];
    f[0] = vn * rho_ln;
#pragma unroll
    for (int d = 0; d < 3; ++d) f[1 + d] = rho_ln * vn * va[d] + p_hat * dir[d];
    f[4] = rho_ln * vn * H;
}

// ------------------------------------------------- mixed form: FP32 flux differencing kernels
// Logarithmic mean of a, b with la = ln a, lb = ln b precomputed per node: the reference's series
// for u = ((a-b)/(a+b))^2 < 1e-2 (navier_stokes.h:494-501), else (a-b)/(ln a - ln b), which is
// the reference's non-series value 0.5(a+b)/(0.5 ln(a/b)/f) written without the per-pair logarithm
// and without its two divisions. Both branches are formed and one is selected (no divergence).
__device__ __forceinline__ float log_mean_f32(float a, float b, float la, float lb)
{
    const float s = a + b, d = a - b;
    const float f = __fdividef(d, s), u = f * f;
    const float F = 1.0f + u * (1.0f / 3 + u * (0.2f + u * (1.0f / 7)));
    const bool series = u < 1e-2f;
    return __fdividef(series ? 0.5f * s : d, series ? F : la - lb);
}

// Chandrashekhar two-point flux (navier_stokes.cc:1510-1542) along an unnormalised direction n:
// the flux is linear in the direction, so F(n) = |n| F(n/|n|) and the volume term
// 2 D_im |nbar| F(nbar/|nbar|) with nbar = (Ja_i + Ja_m)/2 equals D_im F(Ja_i + Ja_m); no
// normalisation is needed. q = {rho, 1/rho, v0, v1, v2, p, beta, ln rho, ln beta, |v|^2};
// hg = 1/(2(gamma-1)).
__device__ __forceinline__ void chandrashekhar_pair_f32(const float qi[10], const float qm[10], const float n[3],
                                                        float hg, float f[5])
{
    const float rho_ln = log_mean_f32(qi[0], qm[0], qi[7], qm[7]);
    const float beta_ln = log_mean_f32(qi[6], qm[6], qi[8], qm[8]);
    const float p_hat = __fdividef(0.5f * (qi[0] + qm[0]), qi[6] + qm[6]);
    const float va0 = 0.5f * (qi[2] + qm[2]), va1 = 0.5f * (qi[3] + qm[3]), va2 = 0.5f * (qi[4] + qm[4]);
    // sum_d (va_d^2 - vsq_d / 2) with vsq_d = (v_i,d^2 + v_m,d^2) / 2
    const float H = __fdividef(hg, beta_ln) + __fdividef(p_hat, rho_ln) + (va0 * va0 + va1 * va1 + va2 * va2) -
                    0.25f * (qi[9] + qm[9]);
    const float vn = va0 * n[0] + va1 * n[1] + va2 * n[2];
    const float rv = rho_ln * vn;
    f[0] = rv;
    f[1] = rv * va0 + p_hat * n[0];
    f[2] = rv * va1 + p_hat * n[1];
    f[3] = rv * va2 + p_hat * n[2];
    f[4] = rv * H;
}

// The same flux for two identical states: the physical flux along n, with the enthalpy
// gamma/(gamma-1) p/rho + |v|^2/2 (the pair formula's value for q_i = q_m). gf = gamma/(gamma-1).
__device__ __forceinline__ void chandrashekhar_same_f32(const float q[10], const float n[3], float gf, float f[5])
{
    const float vn = q[2] * n[0] + q[3] * n[1] + q[4] * n[2];
    const float rv = q[0] * vn;
    f[0] = rv;
    f[1] = rv * q[2] + q[5] * n[0];
    f[2] = rv * q[3] + q[5] * n[1];
    f[3] = rv * q[4] + q[5] * n[2];
    f[4] = rv * (gf * q[5] * q[1] + 0.5f * q[9]);
}

// The same flux for two identical states (the m = i term of the volume sum). log_avg(x, x)
// returns x exactly (x/x = 1, f = 0, series branch, 0.5*(x+x)/1 = x), so skipping the two
// logarithmic means is bitwise identical to chandrashekhar_vol(q, q, ...).
template <class T>
__device__ __forceinline__ void chandrashekhar_vol_same(const T q[7], const T dir[3], T gma, T f[5])
{
    const T beta_ln = q[6];
    const T p_hat = fdiv(T(0.5) * (q[0] + q[0]), q[6] + q[6]);
    const T rho_ln = q[0];
    T va[3], vsq[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        va[d] = T(0.5) * (q[2 + d] + q[2 + d]);
        vsq[d] = T(0.5) * (q[2 + d] * q[2 + d] + q[2 + d] * q[2 + d]);
    }
    T H = fdiv(T(0.5), (gma - 1) * beta_ln) + fdiv(p_hat, rho_ln);
#pragma unroll
    for (int d = 0; d < 3; ++d) H += va[d] * va[d] - T(0.5) * vsq[d];
    T vn = va[0] * dir[0];
    vn += va[1] * dir[1];
    vn += va[2] * dir[2];
    f[0] = vn * rho_ln;
#pragma unroll
    for (int d = 0; d < 3; ++d) f[1 + d] = rho_ln * vn * va[d] + p_hat * dir[d];
    f[4] = rho_ln * vn * H;
}

// Kennedy-Gruber two-point volume flux (navier_stokes.cc:1549-1574); q = {rho,1/rho,v,p,beta},
// plus e per node passed separately.
template <class T>
__device__ __forceinline__ void kennedy_gruber_vol(const T q1[7], const T q2[7], T e1, T e2, const T dir[3], T gma, T f[5])
{
    T va[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) va[d] = T(0.5) * (q1[2 + d] + q2[2 + d]);
    const T ra = T(0.5) * (q1[0] + q2[0]);
    T s1 = q1[2] * q1[2]; s1 += q1[3] * q1[3]; s1 += q1[4] * q1[4];
    T s2 = q2[2] * q2[2]; s2 += q2[3] * q2[3]; s2 += q2[4] * q2[4];
    const T Ea = T(0.5) * (e1 + e2 + T(0.5) * (s1 + s2));
    const T pa = (gma - 1) * T(0.5) * (q1[0] * e1 + q2[0] * e2);
    T vn = va[0] * dir[0];
    vn += va[1] * dir[1];
    vn += va[2] * dir[2];
    f[0] = vn * ra;
#pragma unroll
    for (int d = 0; d < 3; ++d) f[1 + d] = ra * vn * va[d] + pa * dir[d];
    f[4] = vn * (ra * Ea + pa);
}

// Ismail-Roe two-point volume flux (navier_stokes.cc:1590-1617)
template <class T>
__device__ __forceinline__ void ismail_roe_vol(const T c1[5], const T c2[5], const T dir[3], T gma, T f[5])
{
    const T gs = dsqrt(gma);
    const T a1 = dsqrt(gma * get_p(c1, gma) / c1[0]), a2 = dsqrt(gma * get_p(c2, gma) / c2[0]);
    const T z11 = gs / a1, z12 = gs / a2, z51 = c1[0] * a1 / gs, z52 = c2[0] * a2 / gs;
    const T z5ln = log_avg(z51, z52);
    const T rh = T(0.5) * (z11 + z12) * z5ln;
    const T p1h = (z51 + z52) / (z11 + z12);
    const T p2h = T(0.5) * ((gma + 1) * z5ln / log_avg(z11, z12) + (gma - 1) * p1h) / (gma);
    T hh = gma * p2h / ((gma - 1) * rh);
    T vh[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const T v1 = c1[1 + d] / c1[0], v2 = c2[1 + d] / c2[0];
        vh[d] = (z11 * v1 + z12 * v2) / (z11 + z12);
        hh += T(0.5) * (vh[d] * vh[d]);
    }
    T vn = vh[0] * dir[0];
    vn += vh[1] * dir[1];
    vn += vh[2] * dir[2];
    f[0] = rh * vn;
#pragma unroll
    for (int d = 0; d < 3; ++d) f[1 + d] = rh * vh[d] * vn + p1h * dir[d];
    f[4] = rh * vn * hh;
}

// ---------------------------------------------------------------- x-direction surface fluxes

template <class T>
__device__ __forceinline__ void xflux_phys(const T c[5], T gma, T f[5])
{
    const T dir[3] = {T(1), T(0), T(0)};
    inv_flux(c, dir, gma, f);
}

// HLLC with the pressure-based wave speed estimate (navier_stokes.cc:936-1033)
template <class T>
__device__ __forceinline__ void hllc_x(const T l[5], const T r[5], T gma, T f[5])
{
    const T pl = get_p(l, gma), pr = get_p(r, gma);
    const T pmin = (pl < pr) ? pl : pr, pmax = (pl < pr) ? pr : pl;
    const T ul = fdiv(l[1], l[0]), ur = fdiv(r[1], r[0]);
    const T al = dsqrt(fdiv(gma * pl, l[0])), ar = dsqrt(fdiv(gma * pr, r[0]));
    const T p_pvrs = T(0.5) * (pl + pr) - T(0.5) * (ur - ul) * T(0.5) * (l[0] + r[0]) * T(0.5) * (al + ar);
    T ps;
    if (fdiv(pmax, pmin) < T(2) && pmin <= p_pvrs && p_pvrs <= pmax) {
        ps = p_pvrs;
    } else if (p_pvrs < pmin) {
        const T z = (gma - 1) / (T(2) * gma);
        ps = dpow(((al + ar) - (gma - 1) / T(2) * (ur - ul)) / (al / dpow(pl, z) + ar / dpow(pr, z)), T(1) / z);
    } else {
        const T p0 = (p_pvrs > T(0)) ? p_pvrs : T(0);
        const T gl = dsqrt(T(2) / ((gma + 1) * l[0]) / (p0 + (gma - 1) / (gma + 1) * pl));
        const T gr = dsqrt(T(2) / ((gma + 1) * r[0]) / (p0 + (gma - 1) / (gma + 1) * pr));
        ps = (gl * pl + gr * pr - (ur - ul)) / (gl + gr);
    }
    const T ql = (ps <= pl) ? T(1) : dsqrt(T(1) + (gma + 1) / (T(2) * gma) * (ps / pl - T(1)));
    const T qr = (ps <= pr) ? T(1) : dsqrt(T(1) + (gma + 1) / (T(2) * gma) * (ps / pr - T(1)));
    const T sl = ul - al * ql, sr = ur + ar * qr;
    const T s = fdiv(pr - pl + l[1] * (sl - ul) - r[1] * (sr - ur), l[0] * (sl - ul) - r[0] * (sr - ur));
    if (sl > T(0)) {
        xflux_phys(l, gma, f);
    } else if (s > T(0)) {
        const T t = fdiv(sl - ul, sl - s);
        const T ss[5] = {t * l[0], t * l[0] * s, t * l[2], t * l[3], t * (l[4] + (s - ul) * (l[0] * s + fdiv(pl, sl - ul)))};
        T lf[5];
        xflux_phys(l, gma, lf);
#pragma unroll
        for (int v = 0; v < 5; ++v) f[v] = lf[v] + sl * (ss[v] - l[v]);
    } else if (sr > T(0)) {
        const T t = fdiv(sr - ur, sr - s);
        const T ss[5] = {t * r[0], t * r[0] * s, t * r[2], t * r[3], t * (r[4] + (s - ur) * (r[0] * s + fdiv(pr, sr - ur)))};
        T rf[5];
        xflux_phys(r, gma, rf);
#pragma unroll
        for (int v = 0; v < 5; ++v) f[v] = rf[v] + sr * (ss[v] - r[v]);
    } else {
        xflux_phys(r, gma, f);
    }
}

// Rusanov (navier_stokes.cc:1044-1059)
template <class T>
__device__ __forceinline__ void rusanov_x(const T l[5], const T r[5], T gma, T f[5])
{
    T lf[5], rf[5];
    const T al = dsqrt(gma * get_p(l, gma) / l[0]), ar = dsqrt(gma * get_p(r, gma) / r[0]);
    const T ul = l[1] / l[0], ur = r[1] / r[0];
    xflux_phys(l, gma, lf);
    xflux_phys(r, gma, rf);
    const T a = dabs(ul) + al, b = dabs(ur) + ar;
    const T S = (a < b) ? b : a;
#pragma unroll
    for (int v = 0; v < 5; ++v) f[v] = T(0.5) * (lf[v] + rf[v]) - T(0.5) * S * (r[v] - l[v]);
}

// AUSM+-up (navier_stokes.cc:1070-1121, ausm_functions.h:11-88); the reference's
// `alpha = 3/16*(...)` is an integer division and evaluates to 0, which is kept.
template <class T> __device__ __forceinline__ T a_m1p(T M) { return T(0.5) * (M + dabs(M)); }
template <class T> __device__ __forceinline__ T a_m1n(T M) { return T(0.5) * (M - dabs(M)); }
template <class T> __device__ __forceinline__ T a_m2p(T M) { return T(0.25) * (M + 1) * (M + 1); }
template <class T> __device__ __forceinline__ T a_m2n(T M) { return -T(0.25) * (M - 1) * (M - 1); }
template <class T>
__device__ __forceinline__ void ausm_x(const T l[5], const T r[5], T gma, T f[5])
{
    const T pl = get_p(l, gma), pr = get_p(r, gma);
    T vl[3], vr[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) { vl[d] = l[1 + d] / l[0]; vr[d] = r[1 + d] / r[0]; }
    const T Hl = (l[4] + pl) / l[0], Hr = (r[4] + pr) / r[0];
    const T a12 = T(0.5) * (dsqrt(gma * pl / l[0]) + dsqrt(gma * pr / r[0]));
    const T Ml = vl[0] / a12, Mr = vr[0] / a12;
    const T Mavgsq = T(0.5) * (Ml * Ml + Mr * Mr);
    T mm = (Mavgsq > T(0.3) * T(0.3)) ? Mavgsq : T(0.3) * T(0.3);
    mm = (mm < T(1)) ? mm : T(1);
    const T Mo = dsqrt(mm);
    const T fa = Mo * (T(2) - Mo);
    const T alpha = T(0);
    const T m4p = (dabs(Ml) >= T(1)) ? a_m1p(Ml) : a_m2p(Ml) * (T(1) - T(16) * T(0.125) * a_m2n(Ml));
    const T m4n = (dabs(Mr) >= T(1)) ? a_m1n(Mr) : a_m2n(Mr) * (T(1) + T(16) * T(0.125) * a_m2p(Mr));
    const T sg = T(1) - T(1.0) * Mavgsq;
    const T M12 = m4p + m4n - T(0.25) / fa * ((sg > T(0)) ? sg : T(0)) * T(2) * (pr - pl) / (a12 * a12 * (l[0] + r[0]));
    const T pp = (dabs(Ml) >= T(1)) ? a_m1p(Ml) / Ml : a_m2p(Ml) * ((T(2) - Ml) - T(16) * alpha * Ml * a_m2n(Ml));
    const T pn = (dabs(Mr) >= T(1)) ? a_m1n(Mr) / Mr : a_m2n(Mr) * ((-T(2) - Mr) + T(16) * alpha * Mr * a_m2p(Mr));
    const T p12 = pp * pl + pn * pr - T(0.75) * fa * pp * pn * (l[0] + r[0]) * a12 * (vr[0] - vl[0]);
    if (M12 > T(0)) {
        const T m12 = a12 * M12 * l[0];
        f[0] = m12; f[1] = m12 * vl[0] + p12; f[2] = m12 * vl[1]; f[3] = m12 * vl[2]; f[4] = m12 * Hl;
    } else {
        const T m12 = a12 * M12 * r[0];
        f[0] = m12; f[1] = m12 * vr[0] + p12; f[2] = m12 * vr[1]; f[3] = m12 * vr[2]; f[4] = m12 * Hr;
    }
}

// Chandrashekhar surface flux with the blended matrix dissipation (navier_stokes.cc:1250-1318)
template <class T>
__device__ __forceinline__ void chandrashekhar_x(const T l[5], const T r[5], T gma, T fb, T f[5])
{
    const T pl = get_p(l, gma), pr = get_p(r, gma);
    const T betal = T(0.5) * l[0] / pl, betar = T(0.5) * r[0] / pr, beta_ln = log_avg(betal, betar);
    const T p_hat = T(0.5) * (l[0] + r[0]) / (betal + betar);
    const T rho_ln = log_avg(l[0], r[0]);
    T va[3], vsq[3], vl[3], vr[3];
    const T ril = T(1) / l[0], rir = T(1) / r[0];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        vl[d] = l[1 + d] * ril; vr[d] = r[1 + d] * rir;
        va[d] = T(0.5) * (vl[d] + vr[d]); vsq[d] = T(0.5) * (vl[d] * vl[d] + vr[d] * vr[d]);
    }
    T H = T(0.5) / ((gma - 1) * beta_ln) + p_hat / rho_ln;
#pragma unroll
    for (int d = 0; d < 3; ++d) H += va[d] * va[d] - T(0.5) * vsq[d];
    f[0] = rho_ln * va[0];
    f[1] = rho_ln * va[0] * va[0] + p_hat;
    f[2] = rho_ln * va[0] * va[1];
    f[3] = rho_ln * va[0] * va[2];
    f[4] = rho_ln * va[0] * H;
    const T sl = dsqrt(l[0]), sr = dsqrt(r[0]);
    T vi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) vi[d] = T(1) / (sl + sr) * (sl * vl[d] + sr * vr[d]);
    const T Hi = ((l[4] + pl) / sl + (r[4] + pr) / sr) / (sl + sr);
    T vv = vi[0] * vi[0]; vv += vi[1] * vi[1]; vv += vi[2] * vi[2];
    const T a = dsqrt((gma - 1) * (Hi - T(0.5) * vv));
    T K[5][5], Ki[5][5];
    K[0][0] = 1; K[1][0] = vi[0] - a; K[2][0] = vi[1]; K[3][0] = vi[2]; K[4][0] = Hi - vi[0] * a;
    K[0][1] = 1; K[1][1] = vi[0]; K[2][1] = vi[1]; K[3][1] = vi[2]; K[4][1] = T(0.5) * vv;
    K[0][2] = 0; K[1][2] = 0; K[2][2] = 1; K[3][2] = 0; K[4][2] = vi[1];
    K[0][3] = 0; K[1][3] = 0; K[2][3] = 0; K[3][3] = 1; K[4][3] = vi[2];
    K[0][4] = 1; K[1][4] = vi[0] + a; K[2][4] = vi[1]; K[3][4] = vi[2]; K[4][4] = Hi + vi[0] * a;
    const T t = T(1) / (gma - 1);
    Ki[0][0] = Hi + a * (vi[0] - a) * t; Ki[0][1] = -vi[0] - a * t; Ki[0][2] = -vi[1]; Ki[0][3] = -vi[2]; Ki[0][4] = 1;
    Ki[1][0] = T(2) * (T(2) * a * a * t - Hi); Ki[1][1] = T(2) * vi[0]; Ki[1][2] = T(2) * vi[1]; Ki[1][3] = T(2) * vi[2]; Ki[1][4] = -2;
    Ki[2][0] = -T(2) * vi[1] * a * a * t; Ki[2][1] = 0; Ki[2][2] = T(2) * a * a * t; Ki[2][3] = 0; Ki[2][4] = 0;
    Ki[3][0] = -T(2) * vi[2] * a * a * t; Ki[3][1] = 0; Ki[3][2] = 0; Ki[3][3] = T(2) * a * a * t; Ki[3][4] = 0;
    Ki[4][0] = Hi - a * (vi[0] + a) * t; Ki[4][1] = -vi[0] + a * t; Ki[4][2] = -vi[1]; Ki[4][3] = -vi[2]; Ki[4][4] = 1;
    const T factor = T(0.5) * (gma - 1) / (a * a);
    const T ua = dabs(vi[0]), lr = ua + a, l2 = fb * lr + (T(1) - fb) * ua;
    const T eig[5] = {lr, l2, l2, l2, lr};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            T A = 0;
#pragma unroll
            for (int k = 0; k < 5; ++k) A += K[i][k] * eig[k] * (Ki[k][j] * factor);
            f[i] -= T(0.5) * A * (r[j] - l[j]);
        }
    }
}

// Modified Steger-Warming (navier_stokes.cc:1172-1234; Druguet, Candler & Nompelis 2005): split
// fluxes A+ l + A- r, with A+- = K diag(eig+-) K^-1 (the x eigenvector matrices of
// navier_stokes.cc:641-675 and 780-822) at pressure-weighted averages of the two states, the
// eigenvalues smoothed with 0.3 a (navier_stokes.h:464-476). `pos` selects the A+ side: state a
// weighted 1 - w, b weighted w.
template <class T>
__device__ __forceinline__ void msw_side(const T a[5], const T b[5], T w, bool pos, T gma, T A[5][5])
{
    const T pa = get_p(a, gma), pb = get_p(b, gma);
    T v[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = fdiv((T(1) - w) * a[1 + d], a[0]) + fdiv(w * b[1 + d], b[0]);
    const T rho = (T(1) - w) * a[0] + w * b[0], p = (T(1) - w) * pa + w * pb;
    const T c = dsqrt(fdiv(gma * p, rho));
    const T vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const T H = fdiv(gma * p, (gma - 1) * rho) + T(0.5) * vv;
    const T K[5][5] = {{1, 1, 0, 0, 1},
                       {v[0] - c, v[0], 0, 0, v[0] + c},
                       {v[1], v[1], 1, 0, v[1]},
                       {v[2], v[2], 0, 1, v[2]},
                       {H - v[0] * c, T(0.5) * vv, v[1], v[2], H + v[0] * c}};
    const T t = fdiv(T(1), gma - 1);
    T Ki[5][5] = {{H + c * (v[0] - c) * t, -v[0] - c * t, -v[1], -v[2], 1},
                  {2 * (2 * c * c * t - H), 2 * v[0], 2 * v[1], 2 * v[2], -2},
                  {-2 * v[1] * c * c * t, 0, 2 * c * c * t, 0, 0},
                  {-2 * v[2] * c * c * t, 0, 0, 2 * c * c * t, 0},
                  {H - c * (v[0] + c) * t, -v[0] + c * t, -v[1], -v[2], 1}};
    const T factor = fdiv(T(0.5) * (gma - 1), c * c);
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) Ki[i][j] *= factor;
    const T eps = T(0.3) * c;
    T eig[5];
    const T x[3] = {v[0] - c, v[0], v[0] + c};
    T sx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T s = dsqrt(x[k] * x[k] + eps * eps);
        sx[k] = pos ? T(0.5) * (x[k] + s) : T(0.5) * (x[k] - s);
    }
    eig[0] = sx[0];
    eig[1] = eig[2] = eig[3] = sx[1];
    eig[4] = sx[2];
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            T s = 0;
#pragma unroll
            for (int k = 0; k < 5; ++k) s += K[i][k] * eig[k] * Ki[k][j];
            A[i][j] = s;
        }
}

template <class T>
__device__ __forceinline__ void msw_x(const T l[5], const T r[5], T gma, T f[5])
{
    const T pl = get_p(l, gma), pr = get_p(r, gma);
    const T q = fdiv(T(0.5) * (pr - pl), pl < pr ? pl : pr);
    const T w = fdiv(T(0.5), T(1) + q * q);
    T Ap[5][5], An[5][5];
    msw_side(l, r, w, true, gma, Ap);
    msw_side(r, l, w, false, gma, An);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        T s = 0;
#pragma unroll
        for (int j = 0; j < 5; ++j) s += Ap[i][j] * l[j] + An[i][j] * r[j];
        f[i] = s;
    }
}

template <class T>
__device__ __forceinline__ void surf_xflux(const T l[5], const T r[5], T gma, int isf, T fb, T f[5])
{
    switch (isf) {
    case PLENS_ISF_HLLC: hllc_x(l, r, gma, f); return;
    case PLENS_ISF_RUSANOV: rusanov_x(l, r, gma, f); return;
    case PLENS_ISF_AUSM_PLUS_UP: ausm_x(l, r, gma, f); return;
    case PLENS_ISF_RUSANOV_HLLC: {
        T a[5], b[5];
        rusanov_x(l, r, gma, a);
        hllc_x(l, r, gma, b);
#pragma unroll
        for (int v = 0; v < 5; ++v) f[v] = fb * a[v] + (T(1) - fb) * b[v];
        return;
    }
    case PLENS_ISF_RUSANOV_AUSM_PLUS_UP: {
        T a[5], b[5];
        rusanov_x(l, r, gma, a);
        ausm_x(l, r, gma, b);
#pragma unroll
        for (int v = 0; v < 5; ++v) f[v] = fb * a[v] + (T(1) - fb) * b[v];
        return;
    }
    case PLENS_ISF_CHANDRASHEKHAR: chandrashekhar_x(l, r, gma, fb, f); return;
    case PLENS_ISF_MODIFIED_SW: msw_x(l, r, gma, f); return;
    default:
#pragma unroll
        for (int v = 0; v < 5; ++v) f[v] = T(0) / T(0);
        return;
    }
}

// Rotation of both states into the frame whose x axis is the normal, x-flux, rotation back
// (navier_stokes.cc:482-569; Rodrigues matrix, |x cross n| > 1e-3 threshold).
template <class T>
__device__ __forceinline__ void inv_surf_flux(const T o[5], const T nb[5], const T n[3], T gma, int isf, T fb, T f[5])
{
    T m0 = T(0) * n[2] - T(0) * n[1], m1 = T(0) * n[0] - T(1) * n[2], m2 = T(1) * n[1] - T(0) * n[0];
    T M2 = m0 * m0;
    M2 += m1 * m1;
    M2 += m2 * m2;
    const T M = dsqrt(M2);
    T R[3][3];
    if (M > T(1e-3)) {
        m0 = fdiv(m0, M); m1 = fdiv(m1, M); m2 = fdiv(m2, M);
        const T c = T(1) * n[0] + T(0) * n[1] + T(0) * n[2], t = T(1) - c, s = dsqrt(T(1) - c * c);
        R[0][0] = t * m0 * m0 + c;      R[0][1] = t * m0 * m1 - s * m2; R[0][2] = t * m0 * m2 + s * m1;
        R[1][0] = t * m0 * m1 + s * m2; R[1][1] = t * m1 * m1 + c;      R[1][2] = t * m1 * m2 - s * m0;
        R[2][0] = t * m0 * m2 - s * m1; R[2][1] = t * m1 * m2 + s * m0; R[2][2] = t * m2 * m2 + c;
    } else {
        const T dg = (n[0] < T(0)) ? T(-1) : T(1);
        R[0][0] = dg; R[0][1] = 0; R[0][2] = 0;
        R[1][0] = 0; R[1][1] = dg; R[1][2] = 0;
        R[2][0] = 0; R[2][1] = 0; R[2][2] = dg;
    }
    T orr[5], nr[5];
    orr[0] = o[0]; orr[4] = o[4]; nr[0] = nb[0]; nr[4] = nb[4];
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        T a = T(0), b = T(0);
#pragma unroll
        for (int col = 0; col < 3; ++col) {
            a += R[col][row] * o[1 + col];
            b += R[col][row] * nb[1 + col];
        }
        orr[1 + row] = a;
        nr[1 + row] = b;
    }
    T fr[5];
    surf_xflux(orr, nr, gma, isf, fb, fr);
    f[0] = fr[0];
    f[4] = fr[4];
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        T a = T(0);
#pragma unroll
        for (int col = 0; col < 3; ++col) a += R[row][col] * fr[1 + col];
        f[1 + row] = a;
    }
}

// Mixed form, HLLC: the same flux as the rotation of inv_surf_flux + hllc_x, evaluated in the
// original frame. With the frame's x axis e = n (or +-x when |x cross n| <= 1e-3, where the
// reference keeps the identity, navier_stokes.cc:489-521) the rotated states' x velocity is v.e,
// the physical x-flux rotated back is the flux along e, and the HLLC star state rotated back is
// t (rho, rho (v + (s - v.e) e), E + (s - v.e)(rho s + p/(S - v.e))) (navier_stokes.cc:936-1033).
// The wave-speed estimate keeps the reference's PVRS / TRRS / TSRS choice; the side and the
// supersonic cases are selected without branches.
__device__ __forceinline__ void hllc_n_f32(const float l[5], const float r[5], const float nin[3], float gma, float f[5])
{
    float e[3] = {nin[0], nin[1], nin[2]};
    if (!(sqrtf(nin[1] * nin[1] + nin[2] * nin[2]) > 1e-3f)) {  // |x cross n|
        e[0] = (nin[0] < 0.0f) ? -1.0f : 1.0f;
        e[1] = 0.0f;
        e[2] = 0.0f;
    }
    const float ril = __fdividef(1.0f, l[0]), rir = __fdividef(1.0f, r[0]);
    const float ul = (l[1] * e[0] + l[2] * e[1] + l[3] * e[2]) * ril;
    const float ur = (r[1] * e[0] + r[2] * e[1] + r[3] * e[2]) * rir;
    const float pl = (gma - 1.0f) * (l[4] - 0.5f * (l[1] * l[1] + l[2] * l[2] + l[3] * l[3]) * ril);
    const float pr = (gma - 1.0f) * (r[4] - 0.5f * (r[1] * r[1] + r[2] * r[2] + r[3] * r[3]) * rir);
    const float pmin = fminf(pl, pr), pmax = fmaxf(pl, pr);
    const float al = sqrtf(gma * pl * ril), ar = sqrtf(gma * pr * rir);
    const float p_pvrs = 0.5f * (pl + pr) - 0.125f * (ur - ul) * (l[0] + r[0]) * (al + ar);
    float ps;
    if (__fdividef(pmax, pmin) < 2.0f && pmin <= p_pvrs && p_pvrs <= pmax) {
        ps = p_pvrs;
    } else if (p_pvrs < pmin) {
        const float z = __fdividef(gma - 1.0f, 2.0f * gma);
        ps = __powf(__fdividef((al + ar) - 0.5f * (gma - 1.0f) * (ur - ul), al * __powf(pl, -z) + ar * __powf(pr, -z)),
                    __fdividef(1.0f, z));
    } else {
        const float p0 = fmaxf(p_pvrs, 0.0f), ga = __fdividef(2.0f, gma + 1.0f), gb = __fdividef(gma - 1.0f, gma + 1.0f);
        const float gl = sqrtf(__fdividef(ga * ril, p0 + gb * pl)), gr = sqrtf(__fdividef(ga * rir, p0 + gb * pr));
        ps = __fdividef(gl * pl + gr * pr - (ur - ul), gl + gr);
    }
    const float gq = __fdividef(gma + 1.0f, 2.0f * gma);
    const float ql = (ps <= pl) ? 1.0f : sqrtf(1.0f + gq * (__fdividef(ps, pl) - 1.0f));
    const float qr = (ps <= pr) ? 1.0f : sqrtf(1.0f + gq * (__fdividef(ps, pr) - 1.0f));
    const float sl = ul - al * ql, sr = ur + ar * qr;
    const float ml = l[0] * (sl - ul), mr = r[0] * (sr - ur);
    const float s = __fdividef(pr - pl + ml * ul - mr * ur, ml - mr);
    // side: the left state when sl > 0 or s > 0; supersonic when the side's wave has the sign
    const bool left = (sl > 0.0f) || (s > 0.0f);
    const bool super = left ? (sl > 0.0f) : !(sr > 0.0f);
    const float* K = left ? l : r;
    const float uK = left ? ul : ur, pK = left ? pl : pr, SK = left ? sl : sr;
    float FK[5];
    FK[0] = K[0] * uK;
    FK[1] = uK * K[1] + pK * e[0];
    FK[2] = uK * K[2] + pK * e[1];
    FK[3] = uK * K[3] + pK * e[2];
    FK[4] = (K[4] + pK) * uK;
    const float t = __fdividef(SK - uK, SK - s), ds = s - uK;
    float Us[5];
    Us[0] = t * K[0];
    Us[1] = t * (K[1] + K[0] * ds * e[0]);
    Us[2] = t * (K[2] + K[0] * ds * e[1]);
    Us[3] = t * (K[3] + K[0] * ds * e[2]);
    Us[4] = t * (K[4] + ds * (K[0] * s + __fdividef(pK, SK - uK)));
#pragma unroll
    for (int v = 0; v < 5; ++v) f[v] = super ? FK[v] : FK[v] + SK * (Us[v] - K[v]);
}

// mixed-form surface flux: HLLC in the original frame, the other schemes through the rotation
__device__ __forceinline__ void inv_surf_flux_mx(const float o[5], const float nb[5], const float n[3], float gma, int isf,
                                                 float fb, float f[5])
{
    if (isf == PLENS_ISF_HLLC) hllc_n_f32(o, nb, n, gma, f);
    else inv_surf_flux(o, nb, n, gma, isf, fb, f);
}

// viscous flux along a unit direction from the symmetric stress tensor and heat flux stored as
// avars (navier_stokes.cc:586-624)
template <class T>
__device__ __forceinline__ void dif_flux(const T c[5], const T av[9], const T dir[3], T f[5])
{
    const T st[3][3] = {{av[0], av[1], av[2]}, {av[1], av[3], av[4]}, {av[2], av[4], av[5]}};
    T mf[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T a = T(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) a += st[i][j] * dir[j];
        mf[i] = a;
    }
    f[0] = T(0);
    T f4 = T(0);
    const T ri = T(1.0) / c[0];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const T v = c[1 + d] * ri;
        f[1 + d] = mf[d];
        f4 += -av[6 + d] * dir[d] + v * mf[d];
    }
    f[4] = f4;
}

// entropy variables (navier_stokes.h:404-430)
template <class T>
__device__ __forceinline__ void cons_to_entropy(const T c[5], T gma, T e[5])
{
    const T p = get_p(c, gma);
    const T s = dlog(p) - gma * dlog(c[0]);
    const T beta = T(0.5) * c[0] / p;
    const T ri = T(1) / c[0];
    const T v0 = c[1] * ri, v1 = c[2] * ri, v2 = c[3] * ri;
    T vv = v0 * v0;
    vv += v1 * v1;
    vv += v2 * v2;
    e[0] = (gma - s) / (gma - 1) - beta * vv;
    e[1] = T(2) * beta * v0;
    e[2] = T(2) * beta * v1;
    e[3] = T(2) * beta * v2;
    e[4] = T(-2) * beta;
}

}  // namespace plens_gpu
