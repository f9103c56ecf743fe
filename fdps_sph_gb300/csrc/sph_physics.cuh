// Device restatements of the reference's per-particle physics: Wendland C6
// kernel (kernel.h:8-34), EoS lookups (EoS.h:241-247, 394-400 through
// interpolation.h:33-102) and analytic Tillotson.
#pragma once

#include "sph_internal.cuh"

namespace sph {

constexpr double PI_D = 3.141592653589793;         // math::pi = atan(1) * 4 (mathfunc.h:4)
constexpr double WNORM = 1365.0 / 64.0;            // kernel.h:15

// (1365/64) / (H^3 pi) with H = 2.5 h
__device__ __forceinline__ double kernel_norm(double H) { return WNORM / (H * H * H * PI_D); }

// Wendland C6 pieces for s = r / H (kernel.h:8-34), without the kernel
// normalisation: w = W / norm and g = (dW/ds) / norm.  The reference writes
// g = p^7 (p (8 + 50 s + 96 s^2) - 8 (1 + 8 s + 25 s^2 + 32 s^3)) with
// p = 1 - s; expanded, the bracket is exactly -22 s (1 + 7 s + 16 s^2), the
// form used here because it has no cancellation at small s.
__device__ __forceinline__ void wendland_poly(double s, double &w, double &g) {
    const double p = fmax(1.0 - s, 0.0);
    const double poly = 1.0 + s * (8.0 + s * (25.0 + s * 32.0));
    const double p2 = p * p;
    const double p3 = p2 * p;
    const double p7 = p3 * p3 * p;
    w = poly * (p7 * p);
    g = -22.0 * s * (1.0 + s * (7.0 + s * 16.0)) * p7;
}

// a double as a double-float: hi = the nearest float, lo = the nearest float to the remainder
__device__ __forceinline__ void split_df(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

__device__ __forceinline__ void wendland_poly_f(float s, float &w, float &g) {
    const float p = fmaxf(1.0f - s, 0.0f);
    const float poly = 1.0f + s * (8.0f + s * (25.0f + s * 32.0f));
    const float p2 = p * p;
    const float p3 = p2 * p;
    const float p7 = p3 * p3 * p;
    w = poly * (p7 * p);
    g = -22.0f * s * (1.0f + s * (7.0f + s * 16.0f)) * p7;
}

// a double's bit pattern as an integer of the same order: a < b for doubles (neither a NaN)
// exactly when key(a) < key(b), with -0 and +0 both 0 (they compare equal)
__device__ __forceinline__ long long dorder_key(double d) {
    const long long b = __double_as_longlong(d);
    return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}

// std::lower_bound over an ascending axis (no NaN in it).  The comparisons run on the integer
// pipe through dorder_key, with the same outcome as the FP64 comparisons (a NaN v compares false
// with everything: index 0); on this GPU the FP64 pipe is the bound of the EoS kernel.
__device__ __forceinline__ int lower_bound_d(const double *ax, int n, double v) {
    if (v != v) return 0;
    const long long kv = dorder_key(v);
    int lo = 0, len = n;
    while (len > 0) {
        const int half = len >> 1;
        if (dorder_key(ax[lo + half]) < kv) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    return lo;
}

// BilinearInterpolation::interpolate for two planes at once (same bracket)
__device__ __forceinline__ void table_lookup2(const DevMaterial &m, double rho, double u, double &P, double &cs) {
    int li = lower_bound_d(m.rho, m.n_rho, rho);
    int ci = lower_bound_d(m.u, m.n_u, u);
    if (li > m.n_rho - 1) li = m.n_rho - 1;
    if (ci > m.n_u - 1) ci = m.n_u - 1;
    const int64_t nu = m.n_u;
    if (li < m.n_rho - 1 && ci < m.n_u - 1 && li > 0 && ci > 0) {
        const double r0 = m.rho[li - 1], r1 = m.rho[li], u0 = m.u[ci - 1], u1 = m.u[ci];
        const double xi = (rho - r0) / (r1 - r0);
        const double eta = (u - u0) / (u1 - u0);
        const int64_t a = (int64_t)(li - 1) * nu + (ci - 1), b = (int64_t)li * nu + (ci - 1);
        const int64_t c = (int64_t)(li - 1) * nu + ci, d = (int64_t)li * nu + ci;
        const double w00 = (1 - xi) * (1 - eta), w10 = xi * (1 - eta), w01 = (1 - xi) * eta, w11 = xi * eta;
        P = w00 * m.pres[a] + w10 * m.pres[b] + w01 * m.pres[c] + w11 * m.pres[d];
        cs = w00 * m.snds[a] + w10 * m.snds[b] + w01 * m.snds[c] + w11 * m.snds[d];
    } else {
        const int64_t a = (int64_t)li * nu + ci;
        P = m.pres[a];
        cs = m.snds[a];
    }
}

// BilinearInterpolation::interpolate of one plane (EoS_t::Temperature / Entropy:
// columns 2 / 5, EoS.h:254-260, 407-413)
__device__ __forceinline__ double table_lookup1(const DevMaterial &m, const double *plane, double rho, double u) {
    int li = lower_bound_d(m.rho, m.n_rho, rho);
    int ci = lower_bound_d(m.u, m.n_u, u);
    if (li > m.n_rho - 1) li = m.n_rho - 1;
    if (ci > m.n_u - 1) ci = m.n_u - 1;
    const int64_t nu = m.n_u;
    if (li < m.n_rho - 1 && ci < m.n_u - 1 && li > 0 && ci > 0) {
        const double r0 = m.rho[li - 1], r1 = m.rho[li], u0 = m.u[ci - 1], u1 = m.u[ci];
        const double xi = (rho - r0) / (r1 - r0);
        const double eta = (u - u0) / (u1 - u0);
        const double w00 = (1 - xi) * (1 - eta), w10 = xi * (1 - eta), w01 = (1 - xi) * eta, w11 = xi * eta;
        return w00 * plane[(int64_t)(li - 1) * nu + (ci - 1)] + w10 * plane[(int64_t)li * nu + (ci - 1)] +
               w01 * plane[(int64_t)(li - 1) * nu + ci] + w11 * plane[(int64_t)li * nu + ci];
    }
    return plane[(int64_t)li * nu + ci];
}

// analytic Tillotson, same expressions as the oracle's or_tillotson: the branches are the
// reference's P_co / P_ex (EoS.h:91-103) in their operation order; the regime rule (P_co when
// rho >= rho0 or u <= uiv, P_ex when u >= ucv, linear in u between) and the sound speed
// c^2 = dP/drho + P/rho^2 dP/du floored at 1e-2 A/rho0 are this project's definitions
__device__ __forceinline__ void tillotson(const double *p, double rho, double u, double &P, double &cs) {
    const double rho0 = p[0], u0 = p[1], uiv = p[2], ucv = p[3], A = p[4], B = p[5], a = p[6], b = p[7],
                 alpha = p[8], beta = p[9];
    const double eta = rho / rho0;
    const double mu = eta - 1.0;
    const double om = u / u0 / eta / eta + 1.0;   /* operation order of P_co / P_ex, EoS.h:91-103 */
    const double Pc = (a + b / om) * rho * u + A * mu + B * mu * mu;
    const double dPc_drho = (a + b / om) * u + 2.0 * b * u * (om - 1.0) / (om * om) + (A + 2.0 * B * mu) / rho0;
    const double dPc_du = (a + b / om) * rho - rho * b * (om - 1.0) / (om * om);
    double Pv, dPdrho, dPdu;
    if (rho >= rho0 || u <= uiv) {
        Pv = Pc;
        dPdrho = dPc_drho;
        dPdu = dPc_du;
    } else {
        const double z = 1.0 / eta - 1.0;
        const double E1 = exp(-alpha * z);
        const double E2 = exp(-beta * z * z);
        const double Q = b * rho * u / om + A * mu * E1;
        const double Pe = a * rho * u + Q * E2;
        const double dQ = b * u / om + 2.0 * b * u * (om - 1.0) / (om * om) + A / rho0 * E1 +
                          A * mu * alpha * E1 * (z + 1.0) / rho;
        const double dPe_drho = a * u + dQ * E2 + Q * 2.0 * beta * z * (z + 1.0) * E2 / rho;
        const double dPe_du = a * rho + E2 * (b * rho / om - b * rho * (om - 1.0) / (om * om));
        if (u >= ucv) {
            Pv = Pe;
            dPdrho = dPe_drho;
            dPdu = dPe_du;
        } else {
            const double w = ucv - uiv;
            Pv = ((u - uiv) * Pe + (ucv - u) * Pc) / w;
            dPdrho = ((u - uiv) * dPe_drho + (ucv - u) * dPc_drho) / w;
            dPdu = (Pe - Pc + (u - uiv) * dPe_du + (ucv - u) * dPc_du) / w;
        }
    }
    double c2 = dPdrho + Pv / (rho * rho) * dPdu;
    const double c2min = 1.0e-2 * A / rho0;
    if (!(c2 > c2min)) c2 = c2min;
    P = Pv;
    cs = sqrt(c2);
}

__device__ __forceinline__ void eos_eval(const DevMaterial &m, double rho, double u, double &P, double &cs) {
    if (m.kind == 0) {
        table_lookup2(m, rho, u, P, cs);
    } else if (m.kind == 1) {
        tillotson(m.par, rho, u, P, cs);
    } else if (m.kind == 2) {
        const double g = m.par[0];
        P = (g - 1.0) * rho * u;
        cs = sqrt(g * (g - 1.0) * u);
    } else {
        P = nan("");
        cs = nan("");
    }
}

}  // namespace sph
