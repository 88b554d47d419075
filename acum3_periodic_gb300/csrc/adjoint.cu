// adjoint.cu -- hand-written adjoint of the tonal path.
//
// Objective J = sum_obs mean_bins pA^2 (or any J given by dJ/dpA).  Its gradient with
// respect to the surface rows (Cp, positions, normals per element and step) is formed in
// three steps:
//
//  1. forward: the tonal kernels give pA; g[obs][bin] = dJ/dpA (= 2 pA / T).
//  2. adjoint_kernel: one warp per (element, window of 32 lanes), looping over every
//     observer.  Lane l holds the sample of unwrapped step tau = 30 w - 1 + l, so each
//     sample at lanes 1..30 has both of its interpolation intervals inside the window
//     (windows overlap by two lanes and need no carried state; the periodic wrap comes
//     from the unwrapped tau).  Per observer the lane recomputes the forward integrand and
//     observer time of its sample (nothing is stored from the forward), gathers g at the
//     <= 2 bins of its interval (t(tau-1), t(tau)], forms the interval's contributions to
//     dJ/dp and dJ/dt of both end samples (the hat weights and their derivatives), takes
//     its right neighbour's half through one shuffle, and runs the reverse of the
//     integrand by hand.  The 19 cotangents of its step's record fields accumulate in
//     registers over all observers and are written once: no atomics.  The FP32 form
//     (adjoint_kernel_f32) forms the observer time from a per-observer FP64 anchor as the
//     mixed forward does.
//  3. adjoint_chain_kernel: one block per element, FP64: record cotangents -> cotangents of
//     x, ds, n, ndot, V, Vdot, P, Pdot -> through the transposes of the periodic central
//     differences (V = Dx, Vdot = D^2 x, ndot = Dn, Pdot = DP), of make_periodic and of the
//     scalings -> dJ/dCp, dJ/dx, dJ/dn in file coordinates.
//
// Records as the forward builds them (tonal.cu):
//   g0 = x, y, z, dsD   g1 = M(3), M2   g2 = Md(3), ATD   g3 = L(3), Lm   g4 = Ld(3), x.vInf
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "acum_internal.h"
#include "ctx.h"
#include "ptx.h"

namespace acum {

constexpr int kAdjStride = 30;  // new samples per window
constexpr int kCot = 19;        // record-field cotangents per element-step

struct AdjDev {
    const void* rec;  // FP64 record tiles [Epad][nW][5][32][4]
    int E, nW, T, O, nWa;
    const void* obs;  // [O][3]
    const void* g;    // [O][T]
    double a0, alpha, ialpha, vx, vy, vz, dTau, oM, dPsi, kb;
    unsigned tmod;    // ceil(2^32 / T)
    double* cot;      // [E][T][19] FP64
};

template <typename R>
struct V3 {
    R x, y, z;
};

// reciprocal and square root: IEEE in FP64, the fast hardware forms in FP32 (the FP32
// adjoint is compared with the FP64 one, not with the reference)
__device__ __forceinline__ double rcp_(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcp_(float x) { return rcp_ftz(x); }
__device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_(float x) { return x * rsqrt_ftz(x); }

// floor(t / dPsi) as floor(t * (1 / dPsi)), as the forward forms it
__device__ __forceinline__ int bin_floor(double t, double, double idPsi) { return (int)floor(t * idPsi); }
__device__ __forceinline__ int bin_floor(float t, float, float idPsi) { return (int)floorf(t * idPsi); }

// n mod T for 0 <= n < 2^24 by multiply-high with m = ceil(2^32 / T)
__device__ __forceinline__ int wrap_T(int n, int T, unsigned m)
{
    int r = n - (int)__umulhi((unsigned)n, m) * T;
    return r < 0 ? r + T : r;
}

// forward integrand with the intermediates the reverse pass needs
template <typename R>
struct Fwd {
    R dx, dy, dz, c, beta, s, tr, rx, ry, rz, ir, Mr, Mdr, Lr, Ldr, G, qa, K, base, Y, pt, pl, t;
};

// the 20 record fields of (element, step) from the FP64 tiles [element][window][group][32]
// [4], in the adjoint's precision (the FP32 adjoint rounds them once; the mixed form's
// FP32 records hold a reduced field set, so both adjoints read the FP64 ones)
template <typename R>
__device__ __forceinline__ void load_rec(const double* rec, int nW, int e, int step, R* f)
{
    const double* tile = rec + ((size_t)e * nW + step / kWin) * (kGroups * kWin * 4);
    const int lane = step % kWin;
#pragma unroll
    for (int q = 0; q < kGroups; ++q)
#pragma unroll
        for (int c = 0; c < 4; ++c) f[4 * q + c] = (R)tile[((size_t)q * kWin + lane) * 4 + c];
}

template <typename R>
__device__ __forceinline__ Fwd<R> forward(const R* f, R ox, R oy, R oz, const AdjDev& p, int tau)
{
    Fwd<R> a;
    const R vx = (R)p.vx, vy = (R)p.vy, vz = (R)p.vz, a0 = (R)p.a0;
    a.dx = ox - f[0];
    a.dy = oy - f[1];
    a.dz = oz - f[2];
    a.c = a.dx * a.dx + a.dy * a.dy + a.dz * a.dz;
    a.beta = a.dx * vx + a.dy * vy + a.dz * vz;
    a.s = sqrt_(a.beta * a.beta + (R)p.alpha * a.c);
    a.tr = (a.s - a.beta) * (R)p.ialpha;
    a.rx = a.dx - vx * a.tr;
    a.ry = a.dy - vy * a.tr;
    a.rz = a.dz - vz * a.tr;
    const R r = a0 * a.tr;
    a.ir = rcp_(r);
    a.Mr = (f[4] * a.rx + f[5] * a.ry + f[6] * a.rz) * a.ir;
    a.Mdr = (f[8] * a.rx + f[9] * a.ry + f[10] * a.rz) * a.ir;
    a.Lr = (f[12] * a.rx + f[13] * a.ry + f[14] * a.rz) * a.ir;
    a.Ldr = (f[16] * a.rx + f[17] * a.ry + f[18] * a.rz) * a.ir;
    a.G = rcp_((R)1 - a.Mr);
    a.qa = a0 * a.ir;
    a.K = a.Mdr + a.qa * (a.Mr - f[7]);
    a.base = a.ir * a.G * a.G;
    a.Y = a.Ldr + a.qa * (a.Lr - f[15]) + a.Lr * a.G * a.K;
    a.pt = f[11] * a.base * a.G * a.K;
    a.pl = f[3] * a.base * a.Y;
    // observer time [rad] as core.cu:156 forms it
    a.t = ((R)tau * (R)p.dTau + a.tr) * (R)p.oM;
    return a;
}

// reverse of `forward` for dJ/dp (p = pT + pL) = pb and dJ/dt = tb; adds the record
// cotangents into acc[19] (order of the record fields)
template <typename R>
__device__ __forceinline__ void reverse(const R* f, const Fwd<R>& a, R pb, R tb, const AdjDev& p, R* acc)
{
    const R a0 = (R)p.a0, vx = (R)p.vx, vy = (R)p.vy, vz = (R)p.vz;
    // pt = ATD * base * G * K
    R baseb = pb * f[11] * a.G * a.K;
    R Gb = pb * f[11] * a.base * a.K;
    R Kb = pb * f[11] * a.base * a.G;
    acc[11] += pb * a.base * a.G * a.K;
    // pl = dsD * base * Y,  Y = Ldr + qa (Lr - Lm) + Lr G K
    acc[3] += pb * a.base * a.Y;
    baseb += pb * f[3] * a.Y;
    const R Yb = pb * f[3] * a.base;
    R Ldrb = Yb;
    R qab = Yb * (a.Lr - f[15]);
    R Lrb = Yb * (a.qa + a.G * a.K);
    acc[15] -= Yb * a.qa;
    Gb += Yb * a.Lr * a.K;
    Kb += Yb * a.Lr * a.G;
    // base = ir G^2
    R irb = baseb * a.G * a.G;
    Gb += baseb * (R)2 * a.ir * a.G;
    // K = Mdr + qa (Mr - M2)
    R Mdrb = Kb;
    qab += Kb * (a.Mr - f[7]);
    R Mrb = Kb * a.qa;
    acc[7] -= Kb * a.qa;
    // qa = a0 ir
    irb += qab * a0;
    // G = 1/(1 - Mr)
    Mrb += Gb * a.G * a.G;
    // the four projections X.r_hat = (X . rv) ir
    R rvx = 0, rvy = 0, rvz = 0;
    const R r_len = a0 * a.tr;
    auto proj = [&](int i0, R sb, R val) {
        acc[i0] += sb * a.ir * a.rx;
        acc[i0 + 1] += sb * a.ir * a.ry;
        acc[i0 + 2] += sb * a.ir * a.rz;
        rvx += sb * a.ir * f[i0];
        rvy += sb * a.ir * f[i0 + 1];
        rvz += sb * a.ir * f[i0 + 2];
        irb += sb * val * r_len;  // (X . rv) = val / ir
    };
    proj(4, Mrb, a.Mr);
    proj(8, Mdrb, a.Mdr);
    proj(12, Lrb, a.Lr);
    proj(16, Ldrb, a.Ldr);
    // ir = 1 / (a0 tr), t = (tau dTau + tr) oM
    R trb = -irb * a.ir * a.ir * a0 + tb * (R)p.oM;
    // rv = d - v tr
    R dxb = rvx, dyb = rvy, dzb = rvz;
    trb -= rvx * vx + rvy * vy + rvz * vz;
    // tr = (s - beta) / alpha,  s = sqrt(beta^2 + alpha c)
    const R sb = trb * (R)p.ialpha;
    R betab = -trb * (R)p.ialpha;
    const R q2b = sb * rcp_((R)2 * a.s);
    betab += q2b * (R)2 * a.beta;
    const R cb = q2b * (R)p.alpha;
    dxb += betab * vx + cb * (R)2 * a.dx;
    dyb += betab * vy + cb * (R)2 * a.dy;
    dzb += betab * vz + cb * (R)2 * a.dz;
    // d = obs - x
    acc[0] -= dxb;
    acc[1] -= dyb;
    acc[2] -= dzb;
}

template <typename R>
__global__ void __launch_bounds__(128) adjoint_kernel(AdjDev p)
{
    const int warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp_g >= p.E * p.nWa) return;  // warp-uniform
    const int e = warp_g / p.nWa, w = warp_g % p.nWa;
    const int tau = kAdjStride * w - 1 + lane;  // unwrapped step of this lane's sample
    const int step = tau < 0 ? tau + p.T : (tau >= p.T ? tau - p.T : tau);
    const bool owner = lane >= 1 && lane <= kAdjStride && tau >= 0 && tau < p.T;
    R f[20];
    load_rec<R>(reinterpret_cast<const double*>(p.rec), p.nW, e, step, f);
    R acc[kCot];
#pragma unroll
    for (int k = 0; k < kCot; ++k) acc[k] = 0;
    const R* obs = reinterpret_cast<const R*>(p.obs);
    const R* gg = reinterpret_cast<const R*>(p.g);
    const R dPsi = (R)p.dPsi, idPsi = (R)(1.0 / p.dPsi);
    for (int o = 0; o < p.O; ++o) {
        const Fwd<R> a = forward<R>(f, obs[3 * o], obs[3 * o + 1], obs[3 * o + 2], p, tau);
        const R pc = a.pt + a.pl;
        const R tp = __shfl_up_sync(0xffffffffu, a.t, 1);
        const R pp = __shfl_up_sync(0xffffffffu, pc, 1);
        // interval (t(tau-1), t(tau)] of this lane: bins n with tp < n dPsi <= t
        R rp = 0, lp = 0, rt = 0, lt = 0;
        if (lane >= 1 && a.t > tp) {
            // the bin bounds as the forward forms them: floor(t / dPsi)
            const int n0 = bin_floor(tp, dPsi, idPsi) + 1, n1 = bin_floor(a.t, dPsi, idPsi);
            const R inv = rcp_(a.t - tp);
            const R dp = pc - pp;
            const R* grow = gg + (size_t)o * p.T;
            int idx = n0 >= 0 ? wrap_T(n0, p.T, p.tmod) : ((n0 % p.T) + p.T) % p.T;
            // value = p_a + w (p_b - p_a): d J / d p_b = sum g w, d J / d p_a = sum g (1 - w),
            // and with d value / d t(tau) = -dp w / dt, d value / d t(tau-1) = -dp (1 - w) / dt
            // the time derivatives are -(dp / dt) times those sums
            R sg = 0;
            for (int n = n0; n <= n1 && n - n0 < 4; ++n) {
                const R g = grow[idx];
                if (++idx == p.T) idx = 0;
                const R wgt = ((R)n * dPsi - tp) * inv;
                rp += g * wgt;
                sg += g;
            }
            lp = sg - rp;
            rt = -dp * inv * rp;
            lt = -dp * inv * lp;
        }
        const R pb = rp + __shfl_down_sync(0xffffffffu, lp, 1);
        const R tb = rt + __shfl_down_sync(0xffffffffu, lt, 1);
        if (owner) reverse<R>(f, a, pb, tb, p, acc);
    }
    if (owner) {
        double* out = p.cot + ((size_t)e * p.T + step) * kCot;
#pragma unroll
        for (int k = 0; k < kCot; ++k) out[k] = (double)acc[k];
    }
}

// ---------------------------------------------------------------- FP32 adjoint
//
// The FP32 adjoint forms the observer time as the mixed forward does (tonal.cu): per
// observer the retarded time t0 of the origin is solved once in FP64 and its observer time
// t0 oM / dPsi split into an integer ki (with a multiple of T >= 2^23) and a fraction kf;
// per sample dt = t - t0 solves the difference of the two retarded-time quadratics,
//     alpha dt^2 + 2 b dt - num = 0,  b = s0 - x.v,  num = |x|^2 - 2 x.P,  P = D0 - t0 v,
// and the sample's observer time in bins is tau + ki + x with x = kf + dt oM / dPsi, so
// FP32 rounding applies to dt only (the FP32 observer time in radians of the plain form
// loses ~6e-5 of a bin).  The reverse pass is the plain one: it needs tr = t0 + dt and
// s = sqrt(beta^2 + alpha c), which equals alpha tr + beta at the root.

// one observer, three 128-bit loads
struct __align__(16) AdjAnchor {
    float t0, s0, kf;   // t0, alpha t0 + D0.v, frac(t0 oM / dPsi)
    int ki;             // round(t0 oM / dPsi) modulo T, plus toff
    float px, py, pz;   // P = D0 - t0 v
    float ox;           // D0
    float oy, oz, pad0, pad1;
};

__global__ void adj_anchor_kernel(const float* __restrict__ obs, int O, AdjDev p, int toff, AdjAnchor* out)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= O) return;
    const double x = obs[3 * o], y = obs[3 * o + 1], z = obs[3 * o + 2];
    const double b0 = x * p.vx + y * p.vy + z * p.vz;
    const double c0 = x * x + y * y + z * z;
    const double s0 = sqrt(b0 * b0 + p.alpha * c0);
    const double t0 = c0 / (s0 + b0);  // = (s0 - b0) / alpha without the cancellation
    const double K = t0 * (p.oM / p.dPsi);
    const double Kr = rint(K);
    AdjAnchor a;
    a.t0 = (float)t0;
    a.s0 = (float)s0;
    a.kf = (float)(K - Kr);
    a.px = (float)(x - t0 * p.vx);
    a.py = (float)(y - t0 * p.vy);
    a.pz = (float)(z - t0 * p.vz);
    a.ki = (int)(Kr - floor(Kr / p.T) * p.T) + toff;
    a.ox = (float)x;
    a.oy = (float)y;
    a.oz = (float)z;
    a.pad0 = a.pad1 = 0.f;
    out[o] = a;
}

constexpr float kRoundA = 12582912.0f;  // 1.5 * 2^23
constexpr int kRoundBitsA = 0x4B400000;

// forward<float> with the anchored retarded time; *xo = the observer-time offset x
__device__ __forceinline__ Fwd<float> forward_anchored(const float* f, float ox, float oy, float oz,
                                                       const AdjAnchor& an, const AdjDev& p, float* xo)
{
    Fwd<float> a;
    const float vx = (float)p.vx, vy = (float)p.vy, vz = (float)p.vz, a0 = (float)p.a0, alpha = (float)p.alpha;
    a.dx = ox - f[0];
    a.dy = oy - f[1];
    a.dz = oz - f[2];
    a.c = 0.f;  // not needed by the reverse pass
    a.beta = a.dx * vx + a.dy * vy + a.dz * vz;
    const float xv = f[0] * vx + f[1] * vy + f[2] * vz;
    const float xx = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    const float xp = f[0] * an.px + f[1] * an.py + f[2] * an.pz;
    const float num = xx - 2.0f * xp;
    const float bp = an.s0 - xv;
    const float q = alpha * num + bp * bp;
    const float den = q * rsqrt_ftz(q) + bp;
    const float dt = num * rcp_ftz(den);
    a.tr = an.t0 + dt;
    a.s = alpha * a.tr + a.beta;
    a.rx = a.dx - vx * a.tr;
    a.ry = a.dy - vy * a.tr;
    a.rz = a.dz - vz * a.tr;
    const float r = a0 * a.tr;
    a.ir = rcp_ftz(r);
    a.Mr = (f[4] * a.rx + f[5] * a.ry + f[6] * a.rz) * a.ir;
    a.Mdr = (f[8] * a.rx + f[9] * a.ry + f[10] * a.rz) * a.ir;
    a.Lr = (f[12] * a.rx + f[13] * a.ry + f[14] * a.rz) * a.ir;
    a.Ldr = (f[16] * a.rx + f[17] * a.ry + f[18] * a.rz) * a.ir;
    a.G = rcp_ftz(1.0f - a.Mr);
    a.qa = a0 * a.ir;
    a.K = a.Mdr + a.qa * (a.Mr - f[7]);
    a.base = a.ir * a.G * a.G;
    a.Y = a.Ldr + a.qa * (a.Lr - f[15]) + a.Lr * a.G * a.K;
    a.pt = f[11] * a.base * a.G * a.K;
    a.pl = f[3] * a.base * a.Y;
    a.t = 0.f;
    *xo = an.kf + dt * (float)p.kb;
    return a;
}

// The FP32 adjoint: as adjoint_kernel<double>, with the anchored observer time.  The
// interval of lane l is (u(tau - 1), u(tau)], in bins relative to tau + ki: (x_a - 1, x_b];
// its bins k(a) + 1 ... k(b), their weights and the derivatives with respect to both ends
// as the forward's deposit forms them (tonal.cu deposit_ring), at most four bins.
__global__ void __launch_bounds__(128) adjoint_kernel_f32(AdjDev p, const AdjAnchor* __restrict__ anc)
{
    const int warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp_g >= p.E * p.nWa) return;  // warp-uniform
    const int e = warp_g / p.nWa, w = warp_g % p.nWa;
    const int tau = kAdjStride * w - 1 + lane;  // unwrapped step of this lane's sample
    const int step = tau < 0 ? tau + p.T : (tau >= p.T ? tau - p.T : tau);
    const bool owner = lane >= 1 && lane <= kAdjStride && tau >= 0 && tau < p.T;
    float f[20];
    load_rec<float>(reinterpret_cast<const double*>(p.rec), p.nW, e, step, f);
    float acc[kCot];
#pragma unroll
    for (int k = 0; k < kCot; ++k) acc[k] = 0.f;
    const float* gg = reinterpret_cast<const float*>(p.g);
    const float idPsi = (float)(1.0 / p.dPsi);
    for (int o = 0; o < p.O; ++o) {
        const AdjAnchor an = anc[o];
        float xb;
        const Fwd<float> a = forward_anchored(f, an.ox, an.oy, an.oz, an, p, &xb);
        const float pc = a.pt + a.pl;
        const float xa = __shfl_up_sync(0xffffffffu, xb, 1);
        const float pp = __shfl_up_sync(0xffffffffu, pc, 1);
        const float ta = __fadd_rd(xa, kRoundA), tb = __fadd_rd(xb, kRoundA);
        const int cnt = __float_as_int(tb) - __float_as_int(ta) + 1;
        const float du = (xb - xa) + 1.0f;
        // the interval's bins n: value = p_a + w (p_b - p_a), w = (n - u_a) / du, so
        // d J / d p_b = sum g w, d J / d p_a = sum g (1 - w), and (d value / d u_b = -dp w / du,
        // d value / d u_a = -dp (1 - w) / du) d J / d u_b = -(dp / du) sum g w, d J / d u_a =
        // -(dp / du) sum g (1 - w)
        float rp = 0.f, lp = 0.f, rt = 0.f, lt = 0.f;
        if (lane >= 1 && du > 0.0f && cnt >= 1) {
            const float inv = rcp_ftz(du);
            const float* grow = gg + (size_t)o * p.T;
            // first bin k(a) + 1 = tau + ki + floor(x_a) (>= 0: ki carries toff)
            const int n0 = tau + an.ki - kRoundBitsA + __float_as_int(ta);
            // (a sample far outside the floor's range gives any n0: reduce it safely)
            int idx = (n0 >= 0 && n0 < (1 << 24)) ? wrap_T(n0, p.T, p.tmod) : ((n0 % p.T) + p.T) % p.T;
            float wgt = ((ta - (kRoundA - 1.0f)) - xa) * inv;  // w at the first bin
            const int nb = cnt < 4 ? cnt : 4;
            float sg = 0.f;
            for (int n = 0; n < nb; ++n) {
                const float g = grow[idx];
                if (++idx == p.T) idx = 0;
                rp = fmaf(g, wgt, rp);
                sg += g;
                wgt += inv;
            }
            lp = sg - rp;
            const float c = -(pc - pp) * inv;
            rt = c * rp;
            lt = c * lp;
        }
        const float pb = rp + __shfl_down_sync(0xffffffffu, lp, 1);
        // d J / d u in bins -> d J / d t in radians (u = t / dPsi)
        const float tbr = (rt + __shfl_down_sync(0xffffffffu, lt, 1)) * idPsi;
        if (owner) reverse<float>(f, a, pb, tbr, p, acc);
    }
    if (owner) {
        double* out = p.cot + ((size_t)e * p.T + step) * kCot;
#pragma unroll
        for (int k = 0; k < kCot; ++k) out[k] = (double)acc[k];
    }
}

// g[o][n] = 2 (pT + pL) / T from the forward sums [o][n][2], and J's terms
__global__ void adj_seed_kernel(const double* __restrict__ acc, int O, int T, double* __restrict__ g64,
                                float* __restrict__ g32, double* __restrict__ jrow)
{
    const int o = blockIdx.x;
    double s = 0.0;
    for (int n = threadIdx.x; n < T; n += blockDim.x) {
        const double pa = acc[((size_t)o * T + n) * 2] + acc[((size_t)o * T + n) * 2 + 1];
        s += pa * pa;
        const double g = 2.0 * pa / T;
        if (g64) g64[(size_t)o * T + n] = g;
        if (g32) g32[(size_t)o * T + n] = (float)g;
    }
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) jrow[o] = red[0] / T;
}

// Record cotangents -> file-level gradients, one block per element, FP64.
struct ChainDev {
    const double* cot;     // [E][T][19]
    const double* fields;  // [E][T][18] from the preprocessing
    int E, T, periodic, lowpass;
    double a0, rho, pscale, cfd, dTau;
    double gauss[13];
    // the surface rows (Cp at column 3), to recompute the low-pass filter's inputs
    const float* raw;
    const long long* raw_off;
    const int *e_surf, *e_local, *e_count;
    double* gcp;  // [E][T]
    double* gx;   // [E][T][3]
    double* gn;   // [E][T][3]
};

// Which input the 3-point median of the preprocessing picks (the forward's expression,
// tonal.cu prep_kernel): 0 = left, 1 = middle, 2 = right neighbour.
__device__ __forceinline__ int med_sel(double l, double m, double r)
{
    double hi = l > m ? l : m;
    hi = hi > r ? hi : r;
    double lo = l < m ? l : m;
    lo = lo < r ? lo : r;
    return (l < hi && l > lo) ? 0 : ((m < hi && m > lo) ? 1 : 2);
}

// Transpose of the periodic 13-tap Gaussian (its weights are symmetric, w[k] = w[12 - k],
// so the transpose is the same stencil): out[q] = sum_k w[k] in[(q + k - 6) mod T].
__device__ __forceinline__ void gauss_t(const double* in, double* out, int T, const double* w)
{
    for (int q = threadIdx.x; q < T; q += blockDim.x) {
        double acc = 0.0;
        for (int k = 0; k < 13; ++k) {
            int t = q + k - 6;
            if (t < 0) t += T;
            else if (t > T - 1) t -= T;
            acc += w[k] * in[t];
        }
        out[q] = acc;
    }
}

// Transpose of the periodic 3-point median over the series x: the cotangent of each
// output goes to the input it selected (the median is a selection, differentiable
// wherever the three inputs are distinct): out[u] = sum of in[t] over t in {u-1, u, u+1}
// whose median picked x[u].
__device__ __forceinline__ void median_t(const double* x, const double* in, double* out, int T)
{
    for (int u = threadIdx.x; u < T; u += blockDim.x) {
        const int um = u == 0 ? T - 1 : u - 1, up = u == T - 1 ? 0 : u + 1;
        const int umm = um == 0 ? T - 1 : um - 1, upp = up == T - 1 ? 0 : up + 1;
        double acc = 0.0;
        if (med_sel(x[umm], x[um], x[u]) == 2) acc += in[um];  // median at u - 1, right input
        if (med_sel(x[um], x[u], x[up]) == 1) acc += in[u];    // median at u, middle input
        if (med_sel(x[u], x[up], x[upp]) == 0) acc += in[up];  // median at u + 1, left input
        out[u] = acc;
    }
}

__global__ void __launch_bounds__(256) adjoint_chain_kernel(ChainDev c)
{
    extern __shared__ double sm[];
    const int T = c.T;
    // per element series of field cotangents: V(3), Vd(3), nd(3), P, Pd
    double* bV = sm;            // [3][T]
    double* bVd = bV + 3 * T;   // [3][T]
    double* bnd = bVd + 3 * T;  // [3][T]
    double* bP = bnd + 3 * T;   // [T]
    double* bPd = bP + T;       // [T]
    double* tmp = bPd + T;      // [3][T]
    const int e = blockIdx.x;
    const double D1 = 1.0 / (4.0 * M_PI * c.a0), ia0 = 1.0 / c.a0;
    const double two_dt = 2.0 * c.dTau;
    // local chain at each step
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const double* k = c.cot + ((size_t)e * T + t) * kCot;
        const double* f = c.fields + ((size_t)e * T + t) * kFields;
        const double n[3] = {f[4], f[5], f[6]}, nd[3] = {f[7], f[8], f[9]}, V[3] = {f[10], f[11], f[12]};
        const double ds = f[3], P = f[16], Pd = f[17];
        const double Vn = V[0] * n[0] + V[1] * n[1] + V[2] * n[2];
        double gV[3], gVd[3], gN[3], gNd[3], gP = 0.0, gPd = 0.0;
        for (int i = 0; i < 3; ++i) {
            // M = V/a0, M2 = |V|^2/a0^2, Md = Vd/a0
            gV[i] = k[4 + i] * ia0 + k[7] * 2.0 * V[i] * ia0 * ia0;
            gVd[i] = k[8 + i] * ia0;
            // ATD = D1 rho (V.n) a0 ds
            gV[i] += k[11] * D1 * c.rho * c.a0 * ds * n[i];
            gN[i] = k[11] * D1 * c.rho * c.a0 * ds * V[i];
            // L = P n, Lm = P (n.V)/a0, Ld = Pd n + P nd
            gN[i] += k[12 + i] * P + k[15] * P * V[i] * ia0 + k[16 + i] * Pd;
            gV[i] += k[15] * P * n[i] * ia0;
            gNd[i] = k[16 + i] * P;
            gP += k[12 + i] * n[i] + k[16 + i] * nd[i];
            gPd += k[16 + i] * n[i];
        }
        gP += k[15] * Vn * ia0;
        for (int i = 0; i < 3; ++i) {
            bV[i * T + t] = gV[i];
            bVd[i * T + t] = gVd[i];
            bnd[i * T + t] = gNd[i];
            // direct position and normal cotangents (positions scaled by CFDscale)
            c.gx[((size_t)e * T + t) * 3 + i] = k[i] * c.cfd;  // completed below
            c.gn[((size_t)e * T + t) * 3 + i] = gN[i];
        }
        bP[t] = gP;
        bPd[t] = gPd;
    }
    __syncthreads();
    // transposes of the periodic central difference: D^T v[k] = (v[k-1] - v[k+1]) / (2 dt)
    auto DT = [&](const double* v, int k) {
        const int km = k == 0 ? T - 1 : k - 1, kp = k == T - 1 ? 0 : k + 1;
        return (v[km] - v[kp]) / two_dt;
    };
    // Vd = D V: bV += D^T bVd
    for (int t = threadIdx.x; t < T; t += blockDim.x)
        for (int i = 0; i < 3; ++i) tmp[i * T + t] = bV[i * T + t] + DT(bVd + i * T, t);
    __syncthreads();
    // V = D x, x scaled by CFDscale
    for (int t = threadIdx.x; t < T; t += blockDim.x)
        for (int i = 0; i < 3; ++i) c.gx[((size_t)e * T + t) * 3 + i] += DT(tmp + i * T, t) * c.cfd;
    // nd = D n
    for (int t = threadIdx.x; t < T; t += blockDim.x)
        for (int i = 0; i < 3; ++i) c.gn[((size_t)e * T + t) * 3 + i] += DT(bnd + i * T, t);
    __syncthreads();
    // Pd = D P (periodic) or the biased form
    if (c.periodic == 1) {
        for (int t = threadIdx.x; t < T; t += blockDim.x) tmp[t] = bP[t] + DT(bPd, t);
    } else {
        // du[0] = 3 c1 - 3 c2 + c3, du[T-1] = 3 c(T-2) - 3 c(T-3) + c(T-4), interior central
        // (mathfunc.cu:142-159); transpose through the interior central differences
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            // weight of du[k] (k interior) after folding the two end rows
            auto w = [&](int k) {
                double v = bPd[k];
                if (k == 1) v += 3 * bPd[0];
                if (k == 2) v += -3 * bPd[0];
                if (k == 3) v += bPd[0];
                if (k == T - 2) v += 3 * bPd[T - 1];
                if (k == T - 3) v += -3 * bPd[T - 1];
                if (k == T - 4) v += bPd[T - 1];
                return v;
            };
            // u[t] appears in du[t-1] (+1/(2dt)) and du[t+1] (-1/(2dt)) for interior rows
            double acc = bP[t];
            if (t - 1 >= 1 && t - 1 <= T - 2) acc += w(t - 1) / two_dt;
            if (t + 1 >= 1 && t + 1 <= T - 2) acc -= w(t + 1) / two_dt;
            tmp[t] = acc;
        }
    }
    __syncthreads();
    if (c.lowpass == 1) {
        // tmp holds dJ/dP of the filtered pressure.  The filter (preprocess.cu:323-333) is
        // two passes of (median, Gaussian) after make_periodic; its inputs are recomputed
        // here from Cp exactly as the preprocessing forms them, and the cotangent goes back
        // through Gaussian^T, median^T, Gaussian^T, median^T.  The series live in the
        // velocity rows, which are free by now.
        double* Pm = bV;         // make_periodic(Cp pscale): the first median's input
        double* Q1 = bV + T;     // first median's output
        double* P1 = bV + 2 * T; // first Gaussian's output: the second median's input
        double* A = bVd;
        double* B = bVd + T;
        const int s = c.e_surf[e], j = c.e_local[e], Es = c.e_count[s];
        const float* base = c.raw + c.raw_off[s];
        for (int t = threadIdx.x; t < T; t += blockDim.x) Pm[t] = (double)base[((size_t)t * Es + j) * 8 + 3] * c.pscale;
        __syncthreads();
        {
            const double p0 = Pm[0], p1 = Pm[1], pm = Pm[T - 2], pn = Pm[T - 1];
            const double g0 = p0 - (p1 - p0);
            const double k2 = pn, k1 = g0, s2 = pn - pm, s1 = p0 - g0;
            const int xm = T;
            const double dd = k1, cc = s1 - s2;
            const double bb = -2.0 * (s1 - s2) / xm - 3.0 * (k1 - k2) / xm / xm;
            const double aa = -bb / xm - (s1 - s2) / xm / xm - (k1 - k2) / xm / xm / xm;
            __syncthreads();
            for (int t = threadIdx.x; t < T; t += blockDim.x) {
                const int i = t + 1;
                const double cub = aa * i * i * i + bb * i * i + cc * i + dd;
                Pm[t] = Pm[t] - (cub - k2);
            }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            const double l = Pm[t == 0 ? T - 1 : t - 1], m = Pm[t], r = Pm[t == T - 1 ? 0 : t + 1];
            const int k = med_sel(l, m, r);
            Q1[t] = k == 0 ? l : (k == 1 ? m : r);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            double acc = 0.0;
            for (int k = 0; k < 13; ++k) {
                int q = t + k - 6;
                if (q < 0) q += T;
                else if (q > T - 1) q -= T;
                acc += c.gauss[k] * Q1[q];
            }
            P1[t] = acc;
        }
        __syncthreads();
        gauss_t(tmp, A, T, c.gauss);  // second Gaussian
        __syncthreads();
        median_t(P1, A, B, T);        // second median
        __syncthreads();
        gauss_t(B, A, T, c.gauss);    // first Gaussian
        __syncthreads();
        median_t(Pm, A, tmp, T);      // first median
        __syncthreads();
    }
    // make_periodic (mathfunc.cu:165-206): P'[k] = P[k] - (cubic(k+1) - k2), the cubic
    // linear in k1 = 2 P0 - P1, k2 = P[T-1], s1 = P1 - P0, s2 = P[T-1] - P[T-2]
    if (threadIdx.x == 0) {
        const double xm = T;
        double sk1 = 0, sk2 = 0, ss1 = 0, ss2 = 0;
        for (int k = 0; k < T; ++k) {
            const double i = k + 1, b = tmp[k];
            // cubic = aa i^3 + bb i^2 + cc i + dd with
            // dd = k1, cc = s1 - s2, bb = -2(s1-s2)/xm - 3(k1-k2)/xm^2,
            // aa = -bb/xm - (s1-s2)/xm^2 - (k1-k2)/xm^3; P' = P - cubic + k2
            const double dbb_ds = -2.0 / xm, dbb_dk = -3.0 / (xm * xm);
            const double daa_ds = -dbb_ds / xm - 1.0 / (xm * xm), daa_dk = -dbb_dk / xm - 1.0 / (xm * xm * xm);
            const double dc_ds = daa_ds * i * i * i + dbb_ds * i * i + i;  // d cubic / d(s1-s2)
            const double dc_dk = daa_dk * i * i * i + dbb_dk * i * i;      // d cubic / d(k1-k2), besides dd
            // P' = P - cubic + k2: d/dk1 = -(dc_dk + 1), d/dk2 = dc_dk + 1, d/ds1 = -dc_ds, d/ds2 = dc_ds
            sk1 += b * (-(dc_dk + 1.0));
            sk2 += b * (dc_dk + 1.0);
            ss1 += b * (-dc_ds);
            ss2 += b * dc_ds;
        }
        // k1 = 2 P0 - P1, s1 = P1 - P0, k2 = P[T-1], s2 = P[T-1] - P[T-2]
        tmp[0] += 2.0 * sk1 - ss1;
        tmp[1] += -sk1 + ss1;
        tmp[T - 1] += sk2 + ss2;
        tmp[T - 2] += -ss2;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < T; t += blockDim.x) c.gcp[(size_t)e * T + t] = tmp[t] * c.pscale;
}

struct AdjState {
    DBuf<double> cot, g64, jrow, gcp, gx, gn;
    DBuf<float> g32;
    DBuf<double> obs64;
    DBuf<AdjAnchor> anc;
};

static AdjState* adj_state(acum_ctx* c)
{
    if (!c->adj_state) c->adj_state = new AdjState();
    return reinterpret_cast<AdjState*>(c->adj_state);
}

void release_adj_state(acum_ctx* c)
{
    if (!c->adj_state) return;
    AdjState* s = adj_state(c);
    s->cot.release(); s->g64.release(); s->jrow.release(); s->gcp.release(); s->gx.release(); s->gn.release();
    s->g32.release(); s->obs64.release(); s->anc.release();
    delete s;
    c->adj_state = nullptr;
}

}  // namespace acum

using namespace acum;

#define CKA(call)                                              \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

extern "C" int acum_tonal_adjoint(acum_ctx* ctx, int precision, const double* dJ_dpA, double* J, double* g_cp,
                                  double* g_x, double* g_n)
{
    acum::NvtxRange nvtx_range_("acum_tonal_adjoint");
    if (!ctx) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    if (precision != ACUM_PLAIN_FP64 && precision != ACUM_MIXED) return fail(ctx, ACUM_ERR_INVALID, "precision");
    DeviceGuard gd(ctx->device);
    AdjState* s = adj_state(ctx);
    const int T = ctx->T, O = ctx->nobs;
    const long long E = ctx->E;
    const bool f64 = precision == ACUM_PLAIN_FP64;
    ctx->begin_run();
    // forward; both adjoints read the FP64 records, and the FP64 fields feed the chain
    // kernel
    int rc = ctx->ensure_prep(true, !f64, true);
    if (rc) return rc;
    const size_t n = (size_t)T * O;
    CKA(ctx->d_out.ensure(3 * n));
    rc = ctx->run_tonal(precision, ctx->d_out.p, ctx->d_out.p + n, ctx->d_out.p + 2 * n);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    CKA(s->jrow.ensure(O));
    CKA(s->g64.ensure(n));
    CKA(s->g32.ensure(n));
    adj_seed_kernel<<<O, 256, 0, st>>>(ctx->d_acc.p, O, T, s->g64.p, s->g32.p, s->jrow.p);
    if (dJ_dpA) {
        // caller's cotangent [T][O] -> [O][T]
        std::vector<double> gt(n);
        for (int t = 0; t < T; ++t)
            for (int o = 0; o < O; ++o) gt[(size_t)o * T + t] = dJ_dpA[(size_t)t * O + o];
        std::vector<float> g32(n);
        for (size_t i = 0; i < n; ++i) g32[i] = (float)gt[i];
        CKA(cudaMemcpyAsync(s->g64.p, gt.data(), n * 8, cudaMemcpyHostToDevice, st));
        CKA(cudaMemcpyAsync(s->g32.p, g32.data(), n * 4, cudaMemcpyHostToDevice, st));
        CKA(cudaStreamSynchronize(st));
    }
    AdjDev p;
    memset(&p, 0, sizeof(p));
    p.E = (int)E;
    p.nW = ctx->nW;
    p.T = T;
    p.O = O;
    p.nWa = (T + kAdjStride - 1) / kAdjStride;
    p.a0 = ctx->in.a0;
    p.vx = ctx->der.vinf[0];
    p.vy = ctx->der.vinf[1];
    p.vz = ctx->der.vinf[2];
    p.alpha = p.a0 * p.a0 - (p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
    p.ialpha = 1.0 / p.alpha;
    p.dTau = ctx->der.dTau;
    p.oM = ctx->der.oM;
    p.dPsi = ctx->der.dPsi;
    p.tmod = (unsigned)((0x100000000ull + (unsigned long long)ctx->T - 1) / (unsigned long long)ctx->T);
    CKA(s->cot.ensure((size_t)E * T * kCot));
    p.cot = s->cot.p;
    const long long warps = E * p.nWa;
    const int blocks = (int)((warps * 32 + 127) / 128);
    CKA(cudaEventRecord(ctx->ev[EV_ADJ0], st));
    if (f64) {
        p.rec = ctx->d_rec64.p;
        p.obs = ctx->d_obs64.p;
        p.g = s->g64.p;
        adjoint_kernel<double><<<blocks, 128, 0, st>>>(p);
    } else {
        p.rec = ctx->d_rec64.p;
        p.obs = ctx->d_obs32.p;
        p.g = s->g32.p;
        p.kb = p.oM / p.dPsi;
        CKA(s->anc.ensure((size_t)O));
        const int toff = (int)(((1 << 23) + T - 1) / T * T);
        adj_anchor_kernel<<<(O + 127) / 128, 128, 0, st>>>(ctx->d_obs32.p, O, p, toff, s->anc.p);
        adjoint_kernel_f32<<<blocks, 128, 0, st>>>(p, s->anc.p);
    }
    CKA(cudaEventRecord(ctx->ev[EV_ADJ1], st));
    CKA(cudaGetLastError());
    ChainDev c;
    c.cot = s->cot.p;
    c.fields = ctx->d_fields.p;
    c.E = (int)E;
    c.T = T;
    c.periodic = ctx->in.periodic;
    c.lowpass = ctx->in.lowpass;
    gauss_taps(c.gauss);
    c.raw = ctx->d_raw.p;
    c.raw_off = ctx->d_rawoff.p;
    c.e_surf = ctx->d_esurf.p;
    c.e_local = ctx->d_elocal.p;
    c.e_count = ctx->d_ecount.p;
    c.a0 = ctx->in.a0;
    c.rho = ctx->in.rhoRef;
    c.pscale = 0.5 * ctx->in.rhoRef * (ctx->in.Mref * ctx->in.Mref) * (ctx->in.a0 * ctx->in.a0);
    c.cfd = ctx->in.CFDscale;
    c.dTau = ctx->der.dTau;
    CKA(s->gcp.ensure((size_t)E * T));
    CKA(s->gx.ensure((size_t)E * T * 3));
    CKA(s->gn.ensure((size_t)E * T * 3));
    c.gcp = s->gcp.p;
    c.gx = s->gx.p;
    c.gn = s->gn.p;
    const size_t smem = (size_t)T * 14 * sizeof(double);
    if (smem > 48 * 1024) CKA(cudaFuncSetAttribute(adjoint_chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem));
    adjoint_chain_kernel<<<(int)E, 256, smem, st>>>(c);
    CKA(cudaGetLastError());
    ctx->launches += 3;
    ctx->adj_timed = true;
    std::vector<double> jr(O);
    CKA(cudaMemcpyAsync(jr.data(), s->jrow.p, O * 8, cudaMemcpyDeviceToHost, st));
    if (g_cp) CKA(cudaMemcpyAsync(g_cp, s->gcp.p, (size_t)E * T * 8, cudaMemcpyDeviceToHost, st));
    if (g_x) CKA(cudaMemcpyAsync(g_x, s->gx.p, (size_t)E * T * 24, cudaMemcpyDeviceToHost, st));
    if (g_n) CKA(cudaMemcpyAsync(g_n, s->gn.p, (size_t)E * T * 24, cudaMemcpyDeviceToHost, st));
    rc = ctx->finish_run();
    if (rc) return rc;
    if (J) {
        double j = 0;
        for (int o = 0; o < O; ++o) j += jr[o];
        *J = j;
    }
    return ACUM_OK;
}
