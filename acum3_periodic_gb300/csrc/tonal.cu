// tonal.cu -- sm_103a kernels of the tonal (FW-H thickness + loading) path.
//
//  prep_kernel          preprocess_imper (preprocess.cu:228-413) on the GPU, one block per
//                       element: scaling, make_periodic, optional lowpass, periodic
//                       d/dtau of P, n, x and of the velocity; in FP64 for the plain
//                       form's records, with the geometry in FP32 for the mixed form's
//                       (the pressure path FP64 in both); writes the tiled records the
//                       tonal kernels stream, and the records' largest |x| (the reach test
//                       of the ring kernels).
//  aos_record_kernel    the same records from the reference's AoS arrays (drop-in entry).
//  tonal_mixed_kernel   the hot loop of the mixed form (core.cu:18-259 semantics): one
//                       persistent block per SM takes work items (observer tile, element
//                       chunk) from a counter.  A block owns W observers, one or two per
//                       warp (two share each record load).  Lane = source step inside a
//                       32-step window (windows overlap by one step, so the periodic wrap
//                       is an ordinary interval).  Element stages are moved into shared
//                       memory by bulk copies (cp.async.bulk + mbarrier complete_tx) into a
//                       ring of NS stages shared by the block's warps; the last warp done
//                       with a stage refills it.  Each lane evaluates the Farassat-1A
//                       integrand and the observer time of its step; the periodic
//                       hat-function binning of core.cu:166-231 is done as its equivalent,
//                       the piecewise-linear interpolation of the retarded-time signal onto
//                       the bin grid: lane tau fills the bins in (t(tau-1), t(tau)] from
//                       its own sample and its left neighbour's (one warp shuffle), so lanes
//                       never collide and each warp adds into its own observers' bins in
//                       shared memory with plain read-modify-writes -- no atomics.  The bins
//                       of an observer are a sliding ring of 512 slots (1024 or 2048 for
//                       long periods) flushed into the FP64 sums window by window, or whole
//                       rows of the period for records that reach too far for every ring.
//  tonal_batch_kernel   the same work items of many decks in one persistent launch.
//  tonal_f64_kernel     the plain FP64 form (whole rows, one observer per warp).
//  finalize_kernel      [obs][bin][2] sums -> pT/pL/pA [bin][obs] (main.cu:123-130 layout).
//
// Precision forms.  FP64: every quantity in double, observer time in radians as the
// reference forms it; matches the reference's FP64 build.  Mixed: the integrand in FP32;
// per observer the retarded time of the origin is solved once in FP64 and its observer
// time split into an integer bin and a fraction, and each sample's observer-time offset
// from it comes from the difference of the two retarded-time quadratics in FP32 (every
// term of the size of the source's offset from the origin); bin sums in FP32 in shared
// memory over one work item (at most 512 elements; the ring flushes each bin once the
// windows that reach it have passed), then added into FP64 sums in global memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "acum_internal.h"
#include "ptx.h"

namespace acum {

// ------------------------------------------------------------------ helpers

constexpr int kMaxStages = 8;

struct dbl4 {
    double x, y, z, w;
};

// ------------------------------------------------------------ preprocessing

// One block per element.  Shared memory: the element's rows [T][8] as float, then two
// double series (P and a ping-pong buffer for the filters).
// R = double: the FP64 records and the fields; R = float: the FP32 records (the mixed
// form's preprocessing) with the geometry in FP32.  The pressure path (scaling,
// make_periodic, low-pass, time derivative) is FP64 in both: its central difference of
// nearby values loses ~1e-4 of the derivative in FP32.  The FP32 second difference of
// the positions uses error-free differences (each difference's rounding error carried),
// so that it is exact to one rounding.
template <typename R>
__global__ void __launch_bounds__(256) prep_kernel(PrepArgs a)
{
    extern __shared__ __align__(16) unsigned char sm[];
    const int T = a.T;
    float* rows = reinterpret_cast<float*>(sm);                  // [T][8]
    double* P = reinterpret_cast<double*>(sm + (size_t)T * 32);  // [T]
    double* Q = P + T;                                           // [T]
    const int e = blockIdx.x;
    const int s = a.e_surf[e];
    const int j = a.e_local[e];
    const int Es = a.e_count[s];
    const float* base = a.raw + a.raw_off[s];
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const float4* src = reinterpret_cast<const float4*>(base + ((size_t)t * Es + j) * 8);
        float4 v0 = src[0], v1 = src[1];
        float4* dst = reinterpret_cast<float4*>(rows + (size_t)t * 8);
        dst[0] = v0;
        dst[1] = v1;
    }
    __syncthreads();
    // scaled pressure (preprocess.cu:279)
    for (int t = threadIdx.x; t < T; t += blockDim.x) P[t] = (double)rows[t * 8 + 3] * a.pscale;
    __syncthreads();
    // make_periodic (mathfunc.cu:165-206): cubic through the end mismatch
    {
        double p0 = P[0], p1 = P[1], pm = P[T - 2], pn = P[T - 1];
        const double g0 = p0 - (p1 - p0);  // linear extrapolation before the first sample
        double k2 = pn, k1 = g0, s2 = pn - pm, s1 = p0 - g0;
        int xm = T;
        double dd = k1, cc = s1 - s2;
        double bb = -2.0 * (s1 - s2) / xm - 3.0 * (k1 - k2) / xm / xm;
        double aa = -bb / xm - (s1 - s2) / xm / xm - (k1 - k2) / xm / xm / xm;
        __syncthreads();
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            int i = t + 1;
            double cub = aa * i * i * i + bb * i * i + cc * i + dd;
            P[t] = P[t] - (cub - k2);
        }
        __syncthreads();
    }
    if (a.lowpass == 1) {
        // two passes of (3-point periodic median, 13-tap periodic Gaussian)
        // (preprocess.cu:323-333, mathfunc.cu:208-341 and 375-421)
        for (int pass = 0; pass < 2; ++pass) {
            for (int t = threadIdx.x; t < T; t += blockDim.x) {
                double l = P[t == 0 ? T - 1 : t - 1], m = P[t], r = P[t == T - 1 ? 0 : t + 1];
                double hi = l > m ? l : m;
                hi = hi > r ? hi : r;
                double lo = l < m ? l : m;
                lo = lo < r ? lo : r;
                Q[t] = (l < hi && l > lo) ? l : ((m < hi && m > lo) ? m : r);
            }
            __syncthreads();
            for (int t = threadIdx.x; t < T; t += blockDim.x) {
                double acc = 0.0;
                for (int k = 0; k < 13; ++k) {
                    int q = t + k - 6;
                    if (q < 0) q += T;
                    else if (q > T - 1) q -= T;
                    acc += a.gauss[k] * Q[q];
                }
                P[t] = acc;
            }
            __syncthreads();
        }
    }
    // central differences multiply by 1 / (2 dTau) (one rounding from the quotient)
    const double pi2dt = 1.0 / (2.0 * a.dTau);  // the pressure path's, FP64
    const R i2dt = (R)pi2dt, i4dt2 = (R)(pi2dt * pi2dt);
    const R D1 = (R)(1.0 / (4.0 * M_PI * a.a0)), ia0 = (R)(1.0 / a.a0), cfd = (R)a.cfd;
    const int nW32 = nwin32(T);
    float rad = 0.f;  // the largest |x| of this thread's FP32 records
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const int tm = t == 0 ? T - 1 : t - 1, tp = t == T - 1 ? 0 : t + 1;
        const int tmm = tm == 0 ? T - 1 : tm - 1, tpp = tp == T - 1 ? 0 : tp + 1;
        double Pd64;
        if (a.periodic == 1) {
            Pd64 = (P[tp] - P[tm]) * pi2dt;
        } else {
            // central interior, ends by cubic extrapolation (mathfunc.cu:142-159)
            auto cd = [&](int k) { return (P[k + 1] - P[k - 1]) * pi2dt; };
            if (t == 0) Pd64 = 3 * cd(1) - 3 * cd(2) + cd(3);
            else if (t == T - 1) Pd64 = 3 * cd(T - 2) - 3 * cd(T - 3) + cd(T - 4);
            else Pd64 = cd(t);
        }
        const R Pd = (R)Pd64;
        const float* r0 = rows + (size_t)t * 8;
        const float* rm = rows + (size_t)tm * 8;
        const float* rp = rows + (size_t)tp * 8;
        const float* rmm = rows + (size_t)tmm * 8;
        const float* rpp = rows + (size_t)tpp * 8;
        R x[3], n[3], nd[3], v[3], vd[3];
        for (int c = 0; c < 3; ++c) {
            x[c] = (R)r0[c] * cfd;
            n[c] = (R)r0[5 + c];
            nd[c] = ((R)rp[5 + c] - (R)rm[5 + c]) * i2dt;
            R xp = (R)rp[c] * cfd, xm = (R)rm[c] * cfd;
            R xpp = (R)rpp[c] * cfd, xmm = (R)rmm[c] * cfd;
            v[c] = (xp - xm) * i2dt;
            if constexpr (std::is_same<R, float>::value) {
                // (xpp - x) - (x - xmm), each difference with its rounding error
                const float d1 = xpp - x[c], b1 = d1 - xpp, e1 = (xpp - (d1 - b1)) + (-x[c] - b1);
                const float d2 = x[c] - xmm, b2 = d2 - x[c], e2 = (x[c] - (d2 - b2)) + (-xmm - b2);
                vd[c] = ((d1 - d2) + (e1 - e2)) * i4dt2;
            } else {
                R vp = (xpp - x[c]) * i2dt, vm = (x[c] - xmm) * i2dt;
                vd[c] = (vp - vm) * i2dt;
            }
        }
        const R ds = (R)r0[4] * cfd * cfd;
        const R Pt = (R)P[t];
        if (std::is_same<R, double>::value && a.fields) {
            double* f = a.fields + ((size_t)e * T + t) * kFields;
            f[0] = x[0]; f[1] = x[1]; f[2] = x[2]; f[3] = ds;
            f[4] = n[0]; f[5] = n[1]; f[6] = n[2];
            f[7] = nd[0]; f[8] = nd[1]; f[9] = nd[2];
            f[10] = v[0]; f[11] = v[1]; f[12] = v[2];
            f[13] = vd[0]; f[14] = vd[1]; f[15] = vd[2];
            f[16] = Pt; f[17] = Pd;
        }
        // records
        R rec[20];
        rec[0] = x[0]; rec[1] = x[1]; rec[2] = x[2]; rec[3] = D1 * ds;
        rec[4] = v[0] * ia0; rec[5] = v[1] * ia0; rec[6] = v[2] * ia0;
        rec[7] = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * ia0 * ia0;
        rec[8] = vd[0] * ia0; rec[9] = vd[1] * ia0; rec[10] = vd[2] * ia0;
        rec[11] = D1 * (R)a.rho * (v[0] * n[0] + v[1] * n[1] + v[2] * n[2]) * (R)a.a0 * ds;
        R L[3], Ld[3];
        for (int c = 0; c < 3; ++c) {
            L[c] = Pt * n[c];
            Ld[c] = Pd * n[c] + Pt * nd[c];
        }
        rec[12] = L[0]; rec[13] = L[1]; rec[14] = L[2];
        rec[15] = (L[0] * v[0] + L[1] * v[1] + L[2] * v[2]) * ia0;
        rec[16] = Ld[0]; rec[17] = Ld[1]; rec[18] = Ld[2];
        rec[19] = x[0] * (R)a.vinf[0] + x[1] * (R)a.vinf[1] + x[2] * (R)a.vinf[2];
        const int w = t / kWin, lane = t % kWin;
        const size_t tile = ((size_t)e * a.nW + w) * (kGroups * kWin * 4);
        for (int q = 0; q < kGroups; ++q) {
            const size_t off = tile + ((size_t)q * kWin + lane) * 4;
            if (std::is_same<R, double>::value && a.rec64) {
                double2* d = reinterpret_cast<double2*>(a.rec64 + off);
                d[0] = make_double2((double)rec[4 * q], (double)rec[4 * q + 1]);
                d[1] = make_double2((double)rec[4 * q + 2], (double)rec[4 * q + 3]);
            }
        }
        if (a.rec32) {
            float f32[16];
            rec32_fields<R>(rec, rec[3], rec[11], rec + 4, rec + 8, rec + 12, rec + 16, f32);
            rec32_store(a.rec32, e, nW32, T, t, f32);
            const float r = sqrtf(f32[0] * f32[0] + f32[1] * f32[1] + f32[2] * f32[2]);
            rad = (r > rad || r != r) ? r : rad;  // a NaN distance is kept
        }
    }
    if (a.rec32) note_radius(a.rmax, rad);
}

template <typename R>
static cudaError_t launch_prep_t(const PrepArgs& a, cudaStream_t s)
{
    const size_t smem = (size_t)a.T * 32 + (size_t)a.T * 2 * sizeof(double);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t err = cudaFuncSetAttribute(prep_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        configured = smem;
    }
    prep_kernel<R><<<a.E, 256, smem, s>>>(a);
    return cudaGetLastError();
}

// FP64 when the FP64 records or the fields are asked for, else FP32 (the FP32 records of
// the mixed form alone)
cudaError_t launch_prep(const PrepArgs& a, cudaStream_t s)
{
    return (a.rec64 || a.fields) ? launch_prep_t<double>(a, s) : launch_prep_t<float>(a, s);
}

// records from the reference's AoS arrays; one thread per (element, step)
template <typename S>
__global__ void aos_record_kernel(AosArgs a)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)a.E * a.T) return;
    const int e = (int)(idx / a.T), t = (int)(idx % a.T);
    const S* X = reinterpret_cast<const S*>(a.X) + a.xoff[e] + (size_t)t * 4;
    const S* N = reinterpret_cast<const S*>(a.N) + a.noff[e] + (size_t)t * 6;
    const S* V = reinterpret_cast<const S*>(a.V) + a.voff[e] + (size_t)t * 6;
    const S* PR = reinterpret_cast<const S*>(a.PR) + a.proff[e] + (size_t)t * 2;
    const double D1 = 1.0 / (4.0 * M_PI * a.a0), ia0 = 1.0 / a.a0;
    double x[3] = {(double)X[0], (double)X[1], (double)X[2]}, ds = (double)X[3];
    double n[3] = {(double)N[0], (double)N[1], (double)N[2]}, nd[3] = {(double)N[3], (double)N[4], (double)N[5]};
    double v[3] = {(double)V[0], (double)V[1], (double)V[2]}, vd[3] = {(double)V[3], (double)V[4], (double)V[5]};
    double Pt = (double)PR[0], Pd = (double)PR[1];
    double rec[20];
    rec[0] = x[0]; rec[1] = x[1]; rec[2] = x[2]; rec[3] = D1 * ds;
    rec[4] = v[0] * ia0; rec[5] = v[1] * ia0; rec[6] = v[2] * ia0;
    rec[7] = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * ia0 * ia0;
    rec[8] = vd[0] * ia0; rec[9] = vd[1] * ia0; rec[10] = vd[2] * ia0;
    rec[11] = D1 * a.rho * (v[0] * n[0] + v[1] * n[1] + v[2] * n[2]) * a.a0 * ds;
    for (int c = 0; c < 3; ++c) {
        rec[12 + c] = Pt * n[c];
        rec[16 + c] = Pd * n[c] + Pt * nd[c];
    }
    rec[15] = (rec[12] * v[0] + rec[13] * v[1] + rec[14] * v[2]) * ia0;
    rec[19] = x[0] * a.vinf[0] + x[1] * a.vinf[1] + x[2] * a.vinf[2];
    const int w = t / kWin, lane = t % kWin;
    const size_t tile = ((size_t)e * a.nW + w) * (kGroups * kWin * 4);
    for (int q = 0; q < kGroups; ++q) {
        const size_t off = tile + ((size_t)q * kWin + lane) * 4;
        if (a.rec64) {
            double2* d = reinterpret_cast<double2*>(a.rec64 + off);
            d[0] = make_double2(rec[4 * q], rec[4 * q + 1]);
            d[1] = make_double2(rec[4 * q + 2], rec[4 * q + 3]);
        }
    }
    if (a.rec32) {
        float f32[16];
        rec32_fields<double>(rec, rec[3], rec[11], rec + 4, rec + 8, rec + 12, rec + 16, f32);
        rec32_store(a.rec32, e, nwin32(a.T), a.T, t, f32);
        note_radius(a.rmax, sqrtf(f32[0] * f32[0] + f32[1] * f32[1] + f32[2] * f32[2]));
    }
}

cudaError_t launch_aos_records(const AosArgs& a, cudaStream_t s)
{
    long long n = (long long)a.E * a.T;
    int blocks = (int)((n + 255) / 256);
    if (a.is_double) aos_record_kernel<double><<<blocks, 256, 0, s>>>(a);
    else aos_record_kernel<float><<<blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// ------------------------------------------------------------- tonal kernel

struct __align__(16) SmpF {
    int k;      // observer time in bins u = k + f: k = floor(u)
    float f;    // u - k in [0, 1] (NaN: the observer time is out of range)
    float pt, pl;
};

// A sample of the ring kernel: observer time in bins u = tau + ki + x (ki the observer's
// anchor, |x| bounded by the reach, ring_ok), from which the deposit takes the floor and
// the fraction itself
struct SmpR {
    float x;
    float pt, pl;
};

struct SmpD {
    int nb;     // floor(t / dPsi), as floor(t * (1 / dPsi))
    double t;   // observer time [rad]
    double pt, pl;
};

__device__ __forceinline__ SmpD sample_f64(const dbl4& g0, const dbl4& g1, const dbl4& g2, const dbl4& g3,
                                           const dbl4& g4, double ox, double oy, double oz, const KParams& p, int tau,
                                           double idPsi)
{
    const double dx = ox - g0.x, dy = oy - g0.y, dz = oz - g0.z;
    const double c = dx * dx + dy * dy + dz * dz;
    const double beta = dx * p.vx + dy * p.vy + dz * p.vz;
    const double s = sqrt(beta * beta + p.alpha * c);
    const double tr = (s - beta) * p.ialpha;
    const double rx = dx - p.vx * tr, ry = dy - p.vy * tr, rz = dz - p.vz * tr;
    const double r = p.a0 * tr;
    const double ir = 1.0 / r;
    const double Mr = (g1.x * rx + g1.y * ry + g1.z * rz) * ir;
    const double Mdr = (g2.x * rx + g2.y * ry + g2.z * rz) * ir;
    const double Lr = (g3.x * rx + g3.y * ry + g3.z * rz) * ir;
    const double Ldr = (g4.x * rx + g4.y * ry + g4.z * rz) * ir;
    const double G = 1.0 / (1.0 - Mr);
    const double qa = p.a0 * ir;
    const double K = Mdr + qa * (Mr - g1.w);
    const double base = ir * G * G;
    SmpD o;
    o.pt = g2.w * base * G * K;
    o.pl = g0.w * base * (Ldr + qa * (Lr - g3.w) + Lr * G * K);
    // observer time (core.cu:156) and its bin floor.  The product by 1 / dPsi may put a
    // time within an ulp of a bin on the other side of it; the interpolated value of that
    // bin is the same to rounding either way (its weight is 0 on one side, 1 on the other,
    // and both intervals share this sample's bin floor)
    o.t = (tau * p.dTau + tr) * p.oM;
    o.nb = (int)floor(o.t * idPsi);
    return o;
}

__device__ __forceinline__ void deposit_f64(double2* acc, int T, const KParams& p, const SmpD& a, const SmpD& b,
                                            double tshift, int nshift, DeviceErr* err)
{
    const double tb = b.t + tshift;
    const int nbb = b.nb + nshift;
    if (!(tb > a.t) || nbb - a.nb > T || nbb - a.nb < 0) {
        flag(err, ACUM_DEVERR_ORDER, &err->order);
        return;
    }
    const double inv = 1.0 / (tb - a.t);
    const double dT = b.pt - a.pt, dL = b.pl - a.pl;
    int idx = (a.nb + 1) % T;
    if (idx < 0) idx += T;
    for (int n = a.nb + 1; n <= nbb; ++n) {
        const double w = (n * p.dPsi - a.t) * inv;
        double2 s = acc[idx];
        s.x += a.pt + w * dT;
        s.y += a.pl + w * dL;
        acc[idx] = s;
        if (++idx == T) idx = 0;
    }
}

template <typename S>
__device__ __forceinline__ S shfl_smp(const S& v, int src);
template <>
__device__ __forceinline__ SmpF shfl_smp<SmpF>(const SmpF& v, int src)
{
    SmpF o;
    o.k = __shfl_sync(0xffffffffu, v.k, src);
    o.f = __shfl_sync(0xffffffffu, v.f, src);
    o.pt = __shfl_sync(0xffffffffu, v.pt, src);
    o.pl = __shfl_sync(0xffffffffu, v.pl, src);
    return o;
}
template <>
__device__ __forceinline__ SmpD shfl_smp<SmpD>(const SmpD& v, int src)
{
    SmpD o;
    o.nb = __shfl_sync(0xffffffffu, v.nb, src);
    o.t = __shfl_sync(0xffffffffu, v.t, src);
    o.pt = __shfl_sync(0xffffffffu, v.pt, src);
    o.pl = __shfl_sync(0xffffffffu, v.pl, src);
    return o;
}
template <typename S>
__device__ __forceinline__ S shfl_up_smp(const S& v);
template <>
__device__ __forceinline__ SmpF shfl_up_smp<SmpF>(const SmpF& v)
{
    SmpF o;
    o.k = __shfl_up_sync(0xffffffffu, v.k, 1);
    o.f = __shfl_up_sync(0xffffffffu, v.f, 1);
    o.pt = __shfl_up_sync(0xffffffffu, v.pt, 1);
    o.pl = __shfl_up_sync(0xffffffffu, v.pl, 1);
    return o;
}
template <>
__device__ __forceinline__ SmpD shfl_up_smp<SmpD>(const SmpD& v)
{
    SmpD o;
    o.nb = __shfl_up_sync(0xffffffffu, v.nb, 1);
    o.t = __shfl_up_sync(0xffffffffu, v.t, 1);
    o.pt = __shfl_up_sync(0xffffffffu, v.pt, 1);
    o.pl = __shfl_up_sync(0xffffffffu, v.pl, 1);
    return o;
}

__host__ __device__ __forceinline__ size_t acc_region_bytes(int W, int T, int acc_bytes)
{
    return ((size_t)W * T * acc_bytes + 127) / 128 * 128;
}

// Adds a warp's bins (and its overflow slot, into bin 0) to the global FP64 sums
// [obs][bin][2] and clears them.  `direct`
// stores instead of adding (the block is the only writer of these sums).
__device__ __forceinline__ void flush_bins(float2* acc, double* g, int T, int lane, bool direct, DeviceErr* err)
{
    __syncwarp();
    for (int n = lane; n < T; n += 32) {
        float2 v = acc[n];
        if (n == 0) {  // the overflow slot: bin 0 of the next period
            v = add2(v, acc[T]);
            acc[T] = make_float2(0.f, 0.f);
        }
        if (!(fabsf(v.x) < 3.0e38f) || !(fabsf(v.y) < 3.0e38f)) flag(err, ACUM_DEVERR_NONFINITE, &err->nonfinite);
        if (direct) {
            reinterpret_cast<double2*>(g)[n] = make_double2((double)v.x, (double)v.y);
        } else if (v.x != 0.0f || v.y != 0.0f) {
            atomicAdd(g + 2 * n, (double)v.x);
            atomicAdd(g + 2 * n + 1, (double)v.y);
        }
        acc[n] = make_float2(0.f, 0.f);
    }
    __syncwarp();
}

// Adds the ring slots of bins b0 .. b0 + nb - 1 (nb <= R; b0 >= 0, with the anchor's
// multiple of T) of a warp's observer row to the global FP64 sums [obs][bin mod T][2] and
// clears them; slot 0 takes the overflow slot R with it.
__device__ __forceinline__ void ring_flush(float2* row, int R, int b0, int nb, double* g, int T, unsigned tm,
                                           int lane, DeviceErr* err)
{
    __syncwarp();
    for (int m = lane; m < nb; m += 32) {
        const int b = b0 + m, sl = b & (R - 1);
        float2 v = row[sl];
        row[sl] = make_float2(0.f, 0.f);
        if (sl == 0) {
            v = add2(v, row[R]);
            row[R] = make_float2(0.f, 0.f);
        }
        if (!(fabsf(v.x) < 3.0e38f) || !(fabsf(v.y) < 3.0e38f)) flag(err, ACUM_DEVERR_NONFINITE, &err->nonfinite);
        if (v.x != 0.0f || v.y != 0.0f) {
            int n = b - (int)__umulhi((unsigned)b, tm) * T;
            n = n < 0 ? n + T : n;
            atomicAdd(g + 2 * n, (double)v.x);
            atomicAdd(g + 2 * n + 1, (double)v.y);
        }
    }
    __syncwarp();
}

// The plain FP64 form.  Same structure as the mixed kernel below (one observer per
// warp, lane = step of a 32-step window, element tiles by bulk copy into an NS-stage
// ring), everything in double; the bins are FP64 in shared memory and written once per
// block at the end.
template <int SE>
__global__ void __launch_bounds__(512, 1) tonal_f64_kernel(const KParams p)
{
    constexpr int kTile = kGroups * kWin * 4;  // reals per (element, window) tile
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_abort;
    __shared__ int s_release[kMaxStages];  // warps done with the stage in each slot
    __shared__ int s_last[kMaxStages];     // last stage issued into each slot (for the drain)

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int W = p.W, T = p.T, NS = p.NS, nW = p.nW;
    double2* acc_all = reinterpret_cast<double2*>(smem);
    // stages start on a 128-byte boundary: they are bulk-copy destinations (16-byte
    // alignment required) read with 128-bit loads
    const size_t stage_off = acc_region_bytes(W, T, 16);
    double* stages = reinterpret_cast<double*>(smem + stage_off);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + stage_off + (size_t)NS * SE * kTile * sizeof(double));
    double2* acc = acc_all + (size_t)warp * T;

    const int item = blockIdx.x;
    const int ot = item % p.obs_tiles, ec = item / p.obs_tiles;
    const int o = ot * W + warp;
    const bool obs_ok = o < p.O;
    const int e0 = ec * p.chunk;
    const int e1 = min(e0 + p.chunk, p.Epad);
    const int ngroups = e1 > e0 ? (e1 - e0) / SE : 0;
    const int N = ngroups * nW;

    for (int i = threadIdx.x; i < W * T; i += blockDim.x) acc_all[i] = make_double2(0.0, 0.0);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&bars[s], 1);
            s_release[s] = 0;
            s_last[s] = -1;
        }
        mbar_fence_init();
        s_abort = 0;
    }
    __syncthreads();

    const double* rec = reinterpret_cast<const double*>(p.rec);
    const uint32_t tile_bytes = kTile * sizeof(double);
    // stage i = (element group i / nW, window i % nW) goes into slot i % NS
    auto issue = [&](int i) {
        const int s = i % NS, g = i / nW, w = i % nW;
        s_last[s] = i;
        mbar_expect_tx(&bars[s], tile_bytes * SE);
        for (int j = 0; j < SE; ++j) {
            const int e = e0 + g * SE + j;
            bulk_g2s(stages + ((size_t)s * SE + j) * kTile, rec + ((size_t)e * nW + w) * kTile, tile_bytes, &bars[s]);
        }
    };
    if (threadIdx.x == 0)
        for (int i = 0; i < NS && i < N; ++i) issue(i);

    const double idPsi = 1.0 / p.dPsi;
    double ox = 0, oy = 0, oz = 0;
    if (obs_ok) {
        ox = p.obs64[3 * o];
        oy = p.obs64[3 * o + 1];
        oz = p.obs64[3 * o + 2];
    }
    SmpD carry[SE], first[SE];

    // counters advanced incrementally (no per-stage integer division)
    int s = 0, w = 0;
    uint32_t par = 0;
    for (int i = 0; i < N; ++i) {
        // the wait result is made warp-uniform before any shuffle below
        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bars[s], par));
        if (!ok) {
            if (lane == 0) {
                s_abort = 1;
                flag(p.err, ACUM_DEVERR_TIMEOUT, &p.err->timeout);
            }
            break;
        }
        if (*(volatile int*)&s_abort) break;
        const int tau = w * kWin + lane;
        const bool valid = tau < T;
        if (obs_ok) {
            const double* st = stages + (size_t)s * SE * kTile;
            SmpD cur[SE];
#pragma unroll
            for (int j = 0; j < SE; ++j) {
                const double* tl = st + (size_t)j * kTile + lane * 4;
                dbl4 gg[kGroups];
#pragma unroll
                for (int q = 0; q < kGroups; ++q) {
                    const double2* pp = reinterpret_cast<const double2*>(tl + q * kWin * 4);
                    double2 u0 = pp[0], u1 = pp[1];
                    gg[q] = dbl4{u0.x, u0.y, u1.x, u1.y};
                }
                cur[j] = sample_f64(gg[0], gg[1], gg[2], gg[3], gg[4], ox, oy, oz, p, tau, idPsi);
            }
            const int last = min(31, T - 1 - w * kWin);
            const bool has_prev = valid && (lane > 0 || w > 0);
#pragma unroll
            for (int j = 0; j < SE; ++j) {
                SmpD prev = shfl_up_smp(cur[j]);
                if (lane == 0) prev = carry[j];
                if (has_prev) deposit_f64(acc, T, p, prev, cur[j], 0.0, 0, p.err);
                if (w == 0) first[j] = shfl_smp(cur[j], 0);
                carry[j] = shfl_smp(cur[j], last);
                if (w == nW - 1 && lane == 0) {
                    // the periodic wrap: (t(T-1), t(0) + period] (core.cu:173-194)
                    SmpD f0 = first[j];
                    const double tw = f0.t + p.lpi;
                    const int nw = (int)floor(tw * idPsi);
                    deposit_f64(acc, T, p, carry[j], f0, p.lpi, nw - f0.nb, p.err);
                }
            }
        }
        // release the slot; the last warp to finish with it refills it with stage i + NS
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            if (atomicAdd(&s_release[s], 1) == nwarps - 1) {
                s_release[s] = 0;
                if (i + NS < N) issue(i + NS);
            }
        }
        if (++s == NS) {
            s = 0;
            par ^= 1u;
        }
        if (++w == nW) w = 0;
    }
    __syncthreads();
    if (s_abort) {
        // drain the copies still in flight before the block exits (bounded waits)
        if (threadIdx.x == 0)
            for (int k = 0; k < NS; ++k)
                if (s_last[k] >= 0) (void)mbar_wait_bounded(&bars[k], (uint32_t)((s_last[k] / NS) & 1));
        __syncthreads();
        return;
    }
    // flush this block's bins
    if (obs_ok) {
        double* gsum = p.acc + (size_t)o * T * 2;
        for (int n = lane; n < T; n += 32) {
            const double2 a = acc[n];
            if (!(fabs(a.x) < 1e300) || !(fabs(a.y) < 1e300)) flag(p.err, ACUM_DEVERR_NONFINITE, &p.err->nonfinite);
            if (p.nchunk == 1) {
                reinterpret_cast<double2*>(gsum)[n] = a;
            } else {
                atomicAdd(gsum + 2 * n, a.x);
                atomicAdd(gsum + 2 * n + 1, a.y);
            }
        }
    }
}

// ------------------------------------------------------------------ mixed form
//
// One warp per observer; lane = source step of a 32-step window; each lane carries SE
// independent samples per stage (one per element of the stage).  The left neighbour of
// lane l's sample comes from one rotating shuffle (lane l-1); lane 0 keeps what it
// received in the previous window (the previous window's lane 31), and the first sample
// of an element stays in lane 0 for the periodic wrap at its end.

// Farassat-1A integrand with U = V and the normal-velocity rates forced to 0
// (core.cu:93-154), rearranged around K = Mdot_r + (a0/r)(Mr - M^2):
//   pThick = ATD/r * G^3 * K
//   pLoad  = dsD/r * G^2 * (Ldot_r + (a0/r)(L_r - L_M) + L_r G K),  G = 1/(1-Mr)
// where the records carry D1 = 1/(4 pi a0) inside ATD and dsD.
//
// Retarded time.  Per observer, the retarded time t0 from the origin is solved once in
// FP64; each sample then solves for t = t0 + dt from the difference of the two retarded-
// time quadratics (core.cu:261-279 form: alpha t^2 + 2 beta t - |d|^2 = 0),
//     alpha dt^2 + 2 b dt - num = 0,   b = s0 + (d - D0).v,
//     num = |d|^2 - |D0|^2 - 2 t0 (d - D0).v = |x|^2 - 2 x.P,   d - D0 = -x,   P = D0 - t0 v
// (D0 = observer, x = source, s0 = alpha t0 + D0.v; P with t0 per observer), whose terms
// are all of the size of the source's offset from the origin rather than of the observer
// distance; the radiation vector is d - v t = P - x - v dt.  The observer time in bins,
// tau + t0 oM/dPsi + dt oM/dPsi, keeps the first part split exactly (FP64) into an integer
// and a fraction, so FP32 rounding applies to dt only.  The floor of the remainder x comes
// from adding 1.5 * 2^23 rounded towards minus infinity (exact for |x| < 2^22: checked per
// sample in the whole-row kernel, bounded by the reach in the ring kernel), leaving a
// fraction in [0, 1]; whole-row bin indices are reduced modulo T by a multiply-high with
// m = ceil(2^32 / T), ring indices by an AND.

constexpr float kRound = 12582912.0f;  // 1.5 * 2^23
constexpr int kRoundBits = 0x4B400000;

struct Anchor {
    float t0, s0, kf;  // t0, alpha t0 + D0.v, frac(t0 * oM / dPsi)
    int ki;            // round(t0 * oM / dPsi) modulo T, plus p.toff
    float px, py, pz;  // D0 - t0 v
};

__device__ __forceinline__ Anchor make_anchor(const KParams& p, float ox, float oy, float oz)
{
    const double x = ox, y = oy, z = oz;
    const double b0 = x * p.vx + y * p.vy + z * p.vz;
    const double c0 = x * x + y * y + z * z;
    const double s0 = sqrt(b0 * b0 + p.alpha * c0);
    const double t0 = c0 / (s0 + b0);  // = (s0 - b0) / alpha without the cancellation
    const double K = t0 * (p.oM / p.dPsi);
    const double Kr = rint(K);
    Anchor a;
    a.t0 = (float)t0;
    a.px = (float)(x - t0 * p.vx);
    a.py = (float)(y - t0 * p.vy);
    a.pz = (float)(z - t0 * p.vz);
    a.s0 = (float)s0;
    a.kf = (float)(K - Kr);
    // bins wrap with period T: the index is kept small, plus the offset p.toff (a multiple
    // of T of at least 2^23) that keeps it non-negative for the modulo
    a.ki = (int)(Kr - floor(Kr / p.T) * p.T) + p.toff;
    return a;
}

// One field group of an element pair as read from the FP32 records: x = both elements'
// field 0, y = field 1, z = field 2, w = field 3.
struct G2 {
    float2 x, y, z, w;
};

__device__ __forceinline__ G2 load_g2(const float* half0)
{
    const float4 lo = *reinterpret_cast<const float4*>(half0);
    const float4 hi = *reinterpret_cast<const float4*>(half0 + kWin * 4);
    G2 g;
    g.x = make_float2(lo.x, lo.y);
    g.y = make_float2(lo.z, lo.w);
    g.z = make_float2(hi.x, hi.y);
    g.w = make_float2(hi.z, hi.w);
    return g;
}

// The samples of one step of an element pair, in packed FP32 (see the comment above for
// the integrand and the anchored retarded time), in two parts: the retarded time and
// the radiation vector from the positions (group 0), then the source terms from the
// other groups.  The tensor-memory form loads the other groups while the first part
// runs.
struct MixedGeom {
    float2 dt, rx, ry, rz, ir;
};

__device__ __forceinline__ MixedGeom mixed_geom(const G2& g0, const Anchor& an, const KParams& p)
{
    // P = D0 - t0 vInf (the anchor's), P - x
    const float2 dx = sub2(f2(an.px), g0.x), dy = sub2(f2(an.py), g0.y), dz = sub2(f2(an.pz), g0.z);
    // x.(-vInf) and |x|^2, recomputed from the position (nv = -vInf); the same for every
    // observer of the element pair
    const float2 xnv = fma2(g0.x, p.nvx2, fma2(g0.y, p.nvy2, mul2(g0.z, p.nvz2)));
    const float2 xx = fma2(g0.x, g0.x, fma2(g0.y, g0.y, mul2(g0.z, g0.z)));
    // anchored retarded time: num = |x|^2 - 2 x.(D0 - t0 vInf)
    const float2 xp = fma2(g0.x, f2(an.px), fma2(g0.y, f2(an.py), mul2(g0.z, f2(an.pz))));
    const float2 num = fma2(f2(-2.0f), xp, xx);
    const float2 bp = add2(f2(an.s0), xnv);
    const float2 q = fma2(p.alpha2, num, mul2(bp, bp));
    const float2 den = fma2(q, make_float2(rsqrt_ftz(q.x), rsqrt_ftz(q.y)), bp);
    MixedGeom m;
    m.dt = mul2(num, make_float2(rcp_ftz(den.x), rcp_ftz(den.y)));
    const float2 tr = add2(f2(an.t0), m.dt);
    // r = D0 - x - vInf (t0 + dt) = P - x - vInf dt
    m.rx = fma2(p.nvx2, m.dt, dx);
    m.ry = fma2(p.nvy2, m.dt, dy);
    m.rz = fma2(p.nvz2, m.dt, dz);
    m.ir = rcp2(mul2(p.a02, tr));
    return m;
}

// g0..g3: the FP32 record groups (x, ATD | M, Ld'x | Md, Ld'y | L', Ld'z).  RANGE: a
// fraction whose x lies outside the floor's range is made NaN (the ring kernel, whose
// decks bound x by the reach, ring_ok, leaves that test out)
template <bool RANGE, typename S>
__device__ __forceinline__ void mixed_source(const MixedGeom& m, const G2& g0, const G2& g1, const G2& g2,
                                             const G2& g3, const Anchor& an, const KParams& p, int tau, S& oa,
                                             S& ob)
{
    const float2 rx = m.rx, ry = m.ry, rz = m.rz, ir = m.ir;
    // |M|^2 and L'.M from the fields they are made of
    const float2 M2 = fma2(g1.x, g1.x, fma2(g1.y, g1.y, mul2(g1.z, g1.z)));
    const float2 Lm = fma2(g3.x, g1.x, fma2(g3.y, g1.y, mul2(g3.z, g1.z)));
    const float2 Mr = mul2(fma2(g1.x, rx, fma2(g1.y, ry, mul2(g1.z, rz))), ir);
    const float2 Mdr = mul2(fma2(g2.x, rx, fma2(g2.y, ry, mul2(g2.z, rz))), ir);
    const float2 Lr = mul2(fma2(g3.x, rx, fma2(g3.y, ry, mul2(g3.z, rz))), ir);
    const float2 Ldr = mul2(fma2(g1.w, rx, fma2(g2.w, ry, mul2(g3.w, rz))), ir);
    const float2 G = rcp2(sub2(f2(1.0f), Mr));
    const float2 qa = mul2(p.a02, ir);
    const float2 K = fma2(qa, sub2(Mr, M2), Mdr);
    const float2 base = mul2(mul2(ir, G), G);
    const float2 pt = mul2(mul2(g0.w, base), mul2(G, K));
    const float2 pl = mul2(base, fma2(mul2(Lr, G), K, fma2(qa, sub2(Lr, Lm), Ldr)));
    // observer time in bins: tau + round(t0 oM/dPsi) + x, x = frac(t0 oM/dPsi) + dt oM/dPsi;
    // outside the floor's range (or not finite) the fraction is NaN, which the deposit
    // rejects (and reports) whatever the integer part holds
    const float2 x = fma2(m.dt, p.kb2, f2(an.kf));
    if constexpr (std::is_same<S, SmpR>::value) {
        oa.x = x.x;
        ob.x = x.y;
    } else {
        const float2 t = __fadd2_rd(x, f2(kRound));
        const float2 fr = sub2(x, add2(t, f2(-kRound)));
        const int kb = tau + an.ki - kRoundBits;
        oa.k = kb + __float_as_int(t.x);
        ob.k = kb + __float_as_int(t.y);
        oa.f = !RANGE || fabsf(x.x) < 4.0e6f ? fr.x : __int_as_float(0x7fc00000);
        ob.f = !RANGE || fabsf(x.y) < 4.0e6f ? fr.y : __int_as_float(0x7fc00000);
    }
    oa.pt = pt.x;
    ob.pt = pt.y;
    oa.pl = pl.x;
    ob.pl = pl.y;
}

// g[q] = group q of the pair's FP32 records
template <bool RANGE, typename S>
__device__ __forceinline__ void sample_mixed2(const G2* g, const Anchor& an, const KParams& p, int tau, S& oa,
                                              S& ob)
{
    const MixedGeom m = mixed_geom(g[0], an, p);
    mixed_source<RANGE>(m, g[0], g[1], g[2], g[3], an, p, tau, oa, ob);
}

// A group as tensor-memory columns 8q .. 8q + 7 of a pair hold it (half 0: f0 e, f0 e+1,
// f1 e, f1 e+1; half 1: the same for fields 2, 3)
__device__ __forceinline__ G2 g2_of(const uint32_t* r)
{
    G2 g;
    g.x = make_float2(__uint_as_float(r[0]), __uint_as_float(r[1]));
    g.y = make_float2(__uint_as_float(r[2]), __uint_as_float(r[3]));
    g.z = make_float2(__uint_as_float(r[4]), __uint_as_float(r[5]));
    g.w = make_float2(__uint_as_float(r[6]), __uint_as_float(r[7]));
    return g;
}

__device__ __forceinline__ int mod_T(int n, int T, unsigned m)
{
    // 0 <= n < 2^25: the multiply-high quotient is floor(n / T) or one more
    int r = n - (int)__umulhi((unsigned)n, m) * T;
    return r < 0 ? r + T : r;
}

__device__ __forceinline__ float small_int_to_float(int v)
{
    return __int_as_float(v + kRoundBits) - kRound;  // exact for |v| < 2^22
}

// A warp's observer row of the whole-row form: the T bins of the period (bin n in slot n
// mod T, by multiply-high with m = ceil(2^32 / T)), then an overflow slot (index T: bin 0
// of the next period, added into bin 0 when the row is flushed) and a scratch slot
// (index T + 1, never read).  (The ring form's rows: deposit_ring.)
//
// Bins n with u(a) < n <= u(b): n = k(a) + 1 ... k(b), the value interpolated between the
// two samples.  For |Mr| < 1 an interval holds at most 2 bins (u(b) - u(a) = 1 - Mr < 2).
// Both are written by every lane without a branch: the first at its slot, the second at
// the slot after it (which may be the overflow slot); a lane with fewer bins adds into
// the scratch slot instead.  The bins of the lanes of a warp are disjoint (observer time
// increases with the step), so only the scratch slot is written by more than one lane.
// A decreasing or non-finite observer time sets `bad` and deposits nothing.  Intervals
// of more than two bins (|Mr| >= 1) set `more`: the caller then adds their other bins
// with deposit_rest.  The integer parts k carry a multiple of T of at least 2^23 (the
// anchor's), which keeps the bin index non-negative.
__device__ __forceinline__ void deposit(float2* acc, int T, unsigned m, const SmpF& a, const SmpF& b, bool active,
                                        unsigned& bad, bool& more)
{
    const int cnt = b.k - a.k;
    const float du = small_int_to_float(cnt) + (b.f - a.f);
    const bool ok = du > 0.0f;  // false for NaN
    bad |= (active && !ok) ? 1u : 0u;
    const bool one = active && ok && cnt >= 1, two = one && cnt >= 2;
    more |= two && cnt > 2;
    // not finite when !ok; both slots are then the scratch slot, which is never read out
    const float inv = rcp_ftz(du);
    const float2 pa = make_float2(a.pt, a.pl), dp = sub2(make_float2(b.pt, b.pl), pa);
    const int idx = mod_T(a.k + 1, T, m);  // used only when `one`
    const float w1 = (1.0f - a.f) * inv;
    const int i1 = one ? idx : T + 1, i2 = two ? idx + 1 : T + 1;
    // i1 != i2 unless both are the scratch slot, so both bins are read before either is
    // written (one shared-memory round trip per sample instead of two in sequence)
    const float2 v1 = acc[i1], v2 = acc[i2];
    acc[i1] = add2(v1, fma2(f2(w1), dp, pa));
    acc[i2] = add2(v2, fma2(f2(w1 + inv), dp, pa));
}

// The bins after the first two of an interval that holds more (see deposit); an interval
// of more than T bins sets `bad` instead.
__device__ __forceinline__ void deposit_rest(float2* acc, int T, unsigned m, const SmpF& a, const SmpF& b,
                                             bool active, unsigned& bad)
{
    const int cnt = b.k - a.k;
    const float du = small_int_to_float(cnt) + (b.f - a.f);
    if (!(active && du > 0.0f && cnt > 2)) return;
    if (cnt > T) {
        bad = 1u;
        return;
    }
    const float inv = rcp_ftz(du);
    const float2 pa = make_float2(a.pt, a.pl), dp = sub2(make_float2(b.pt, b.pl), pa);
    const float w1 = (1.0f - a.f) * inv;
    int i = mod_T(a.k + 1, T, m);
    for (int q = 1; q < cnt; ++q) {
        if (++i >= T) i -= T;
        if (q >= 2) acc[i] = add2(acc[i], fma2(f2(w1 + (float)q * inv), dp, pa));
    }
}

// The ring form of deposit / deposit_rest on SmpR samples, in a row of R slots (bin n in
// slot n mod R, R a power of two, m = R - 1), an overflow slot R (slot 0's bin, added into
// it when the slot is flushed) and a scratch slot R + 1: a = lane l - 1's sample (step
// tau - 1), b = this lane's (step tau); base = tau + ki - 1.5 * 2^23 (as an int), so that the
// first bin of the interval, k(a) + 1 = tau + ki + floor(x_a), is base + the bits of
// x_a + 1.5 * 2^23 rounded down.  The interval's length in bins is 1 + x_b - x_a (= the
// whole-row form's cnt + f_b - f_a) and the weight 1 - f_a = floor(x_a) + 1 - x_a.
__device__ __forceinline__ void deposit_ring(float2* acc, int R, unsigned m, const SmpR& a, const SmpR& b, int base,
                                             bool active, unsigned& bad, bool& more)
{
    const float ta = __fadd_rd(a.x, kRound), tb = __fadd_rd(b.x, kRound);
    const int cnt = __float_as_int(tb) - __float_as_int(ta) + 1;
    const float du = (b.x - a.x) + 1.0f;
    const bool ok = du > 0.0f;  // false for NaN
    bad |= (active && !ok) ? 1u : 0u;
    const bool one = active && ok && cnt >= 1, two = one && cnt >= 2;
    more |= two && cnt > 2;
    // not finite when !ok; both slots are then the scratch slot, which is never read out
    const float inv = rcp_ftz(du);
    const float2 pa = make_float2(a.pt, a.pl), dp = sub2(make_float2(b.pt, b.pl), pa);
    const int idx = (int)((unsigned)(base + __float_as_int(ta)) & m);  // used only when `one`
    const float w1 = ((ta - (kRound - 1.0f)) - a.x) * inv;
    const int i1 = one ? idx : R + 1, i2 = two ? idx + 1 : R + 1;
    const float2 v1 = acc[i1], v2 = acc[i2];
    acc[i1] = add2(v1, fma2(f2(w1), dp, pa));
    acc[i2] = add2(v2, fma2(f2(w1 + inv), dp, pa));
}

__device__ __forceinline__ void deposit_rest_ring(float2* acc, int R, unsigned m, const SmpR& a, const SmpR& b,
                                                  int base, bool active, unsigned& bad)
{
    const float ta = __fadd_rd(a.x, kRound), tb = __fadd_rd(b.x, kRound);
    const int cnt = __float_as_int(tb) - __float_as_int(ta) + 1;
    const float du = (b.x - a.x) + 1.0f;
    if (!(active && du > 0.0f && cnt > 2)) return;
    if (cnt > R) {
        bad = 1u;
        return;
    }
    const float inv = rcp_ftz(du);
    const float2 pa = make_float2(a.pt, a.pl), dp = sub2(make_float2(b.pt, b.pl), pa);
    const float w1 = ((ta - (kRound - 1.0f)) - a.x) * inv;
    int i = (int)((unsigned)(base + __float_as_int(ta)) & m);
    for (int q = 1; q < cnt; ++q) {
        i = (int)((unsigned)(i + 1) & m);
        if (q >= 2) acc[i] = add2(acc[i], fma2(f2(w1 + (float)q * inv), dp, pa));
    }
}

__device__ __forceinline__ SmpR shfl_idx(const SmpR& v, int src)
{
    SmpR o;
    o.x = __shfl_sync(0xffffffffu, v.x, src);
    o.pt = __shfl_sync(0xffffffffu, v.pt, src);
    o.pl = __shfl_sync(0xffffffffu, v.pl, src);
    return o;
}

__device__ __forceinline__ SmpF shfl_idx(const SmpF& v, int src)
{
    SmpF o;
    o.k = __shfl_sync(0xffffffffu, v.k, src);
    o.f = __shfl_sync(0xffffffffu, v.f, src);
    o.pt = __shfl_sync(0xffffffffu, v.pt, src);
    o.pl = __shfl_sync(0xffffffffu, v.pl, src);
    return o;
}

// Block-wide shared state of the mixed kernels besides the dynamic shared memory.
template <int SE, int OPW>
struct __align__(16) MixedShared {
    uint64_t tfull[kMaxStages];  // tensor-memory form: a slot's copy into tensor memory is complete
    int abort;
    int release[kMaxStages];
    int last[kMaxStages];
    int claim[kMaxStages];   // tensor-memory form: warps that reached the slot's stage (the first copies)
    int copied[kMaxStages];  // tensor-memory form: stage of the slot's last copy, -1 = none
    uint32_t tmem;           // tensor-memory form: base address of the block's columns
};

// Tensor-memory form: stage slot s, element pair jp of the stage, occupies the 32 columns
// from tm_col(s, jp) (8 blocks of 4: group q, half h at 4 (2q + h)).
template <int SE>
__device__ __forceinline__ uint32_t tm_col(int s, int jp)
{
    return (uint32_t)((s * (SE / 2) + jp) * 32);
}
constexpr uint32_t kTmemCols = 512;  // NS x SE / 2 x 32 <= 512 for every stage shape the plan allows

// Ring form: the largest distance of a sample's bin from its step plus the anchor's, in
// bins (ring_reach_bins with the records' largest |x|).
__device__ __forceinline__ double ring_reach(const KParams& p)
{
    return ring_reach_bins(__uint_as_float(*p.rmax), p.vx, p.vy, p.vz, p.a0, p.oM / p.dPsi);
}

// One work item of the mixed form: observers [ot*W, ot*W + W) and elements [e0, e1)
// (a multiple of SE) of the deck `p`; each warp evaluates OPW observers on the records it
// loads once.  The dynamic shared memory holds the FP32 bin rows (W rows of nb + 2
// float2: nb = T bins of the period, or the R slots of a ring) followed by the NS-stage
// ring of record stages; `stage_off` is where the stages start (fixed for a launch).
// `gbase` counts the stages the block has consumed before this item, so consecutive
// items of a block continue the mbarrier phases of the same stage ring.  On entry every
// stage slot is free and all bin rows are zero; on return (without abort) the same holds
// again.
//
// A stage holds SE elements' records of one 32-step window (windows overlap by one step:
// lane l of window w is step 31 w + l, up to step T = step 0 of the next period).  Lane
// l >= 1 deposits the interval between its sample and lane l - 1's, so every interval of
// the period, the wrap (T - 1, T] included, is deposited once, by the window that holds
// both its ends.
//
// Whole rows (RING = false): the stages take the windows of an element group in turn, and
// the rows are added into the FP64 sums after the group's last window (every
// `flush_groups` groups).  Ring (RING = true): the stages take every element group of a
// window before the next window.  The bins that window w reaches lie within a span of 31
// + 2 x reach (ring_reach) bins that moves by 31 per window, so each row is a ring of R
// slots (bin n in slot n mod R) and after a window's last group its lowest 31 bins, which
// no later window reaches, are added into the FP64 sums and cleared; the rest at the end
// of the item.
template <int SE, int OPW, bool TM, bool RING>
__device__ __forceinline__ void mixed_item(const KParams& __restrict__ p, int ot, int e0, int e1, unsigned char* smem,
                                           size_t stage_off, MixedShared<SE, OPW>& sh, unsigned& gbase)
{
    constexpr int kTile = kGroups32 * kWin * 4;  // floats per (element, window) of the FP32 records
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int W = p.W;  // observers per block = OPW x warps
    const int T = p.T, NS = p.NS, nW = p.nW32;
    const int nb = RING ? p.ring : T;                                // slots per row
    const unsigned mm = RING ? (unsigned)(p.ring - 1) : p.tmod;      // their index modulus
    float2* acc_all = reinterpret_cast<float2*>(smem);
    float* stages = reinterpret_cast<float*>(smem + stage_off);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + stage_off + (size_t)NS * SE * kTile * sizeof(float));
    const int ngroups = e1 > e0 ? (e1 - e0) / SE : 0;
    const int N = ngroups * nW;
    const unsigned g0 = gbase;

    // stage i: element group and window
    const auto stage_gw = [&](int i, int& g, int& w) {
        if (RING) {
            w = i / ngroups;
            g = i - w * ngroups;
        } else {
            g = i / nW;
            w = i - g * nW;
        }
    };
    // stage = SE / 2 element-pair tiles of one window (2 kTile floats each)
    const float* rec = reinterpret_cast<const float*>(p.rec);
    const uint32_t pair_bytes = 2 * kTile * sizeof(float);
    auto issue = [&](int i) {
        const unsigned gi = g0 + (unsigned)i;
        const int s = (int)(gi % (unsigned)NS);
        int g, w;
        stage_gw(i, g, w);
        sh.last[s] = (int)gi;
        mbar_expect_tx(&bars[s], pair_bytes * (SE / 2));
        for (int jp = 0; jp < SE / 2; ++jp) {
            const int pr = (e0 + g * SE) / 2 + jp;
            bulk_g2s(stages + ((size_t)s * SE + 2 * jp) * kTile, rec + ((size_t)pr * nW + w) * (2 * kTile), pair_bytes,
                     &bars[s]);
        }
    };
    if (threadIdx.x == 0)
        for (int i = 0; i < NS && i < N; ++i) issue(i);

    int o[OPW];
    bool ok_obs[OPW];
    float ox[OPW], oy[OPW], oz[OPW];
    float2* acc[OPW];
    Anchor anc[OPW];
    int lo[OPW];  // ring: the lowest bin window 0 reaches
    const double reach = RING ? ring_reach(p) : 0.0;
#pragma unroll
    for (int q = 0; q < OPW; ++q) {
        o[q] = ot * W + warp * OPW + q;
        ok_obs[q] = o[q] < p.O;
        const int oc = ok_obs[q] ? o[q] : 0;
        ox[q] = p.obs32[3 * oc];
        oy[q] = p.obs32[3 * oc + 1];
        oz[q] = p.obs32[3 * oc + 2];
        acc[q] = acc_all + (size_t)(warp * OPW + q) * (nb + 2);  // nb slots, the overflow and the scratch slot
        anc[q] = make_anchor(p, ox[q], oy[q], oz[q]);
        // a sample at step tau has bin k = tau + ki + floor(x), x >= kf - reach, and lane
        // tau >= 31 w + 1 deposits bins above k(tau - 1)
        lo[q] = RING ? anc[q].ki + (int)floor((double)anc[q].kf - reach) + 1 : 0;
    }
    unsigned bad = 0;
    bool more = false;

    int s = (int)(g0 % (unsigned)NS), since_flush = 0;
    uint32_t par = (g0 / (unsigned)NS) & 1u;
    for (int i = 0; i < N; ++i) {
        bool ok;
        if (TM) {
            // the first warp to reach the stage copies it from shared into tensor memory,
            // once its bulk copies have landed; every warp then waits for that copy
            int c = 0;
            if (lane == 0) c = atomicAdd(&sh.claim[s], 1);
            c = __shfl_sync(0xffffffffu, c, 0);
            if (c == 0 && lane == 0) {
                if (mbar_wait_bounded(&bars[s], par)) {
                    tmem_fence_after();
                    const float* st = stages + (size_t)s * SE * kTile;
                    for (int jp = 0; jp < SE / 2; ++jp)
                        for (int b = 0; b < 2 * kGroups32; ++b)
                            tmem_cp_32x128b_warpx4(sh.tmem + tm_col<SE>(s, jp) + 4u * b,
                                                   smem_desc_plain(st + (size_t)(2 * jp) * kTile + b * kWin * 4, 128, 128));
                    tmem_commit(&sh.tfull[s]);
                    sh.copied[s] = (int)(g0 + (unsigned)i);
                }
            }
            ok = __all_sync(0xffffffffu, mbar_wait_bounded(&sh.tfull[s], par));
            tmem_fence_after();
        } else {
            ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bars[s], par));
        }
        if (!ok) {
            if (lane == 0) {
                sh.abort = 1;
                flag(p.err, ACUM_DEVERR_TIMEOUT, &p.err->timeout);
            }
            break;
        }
        if (*(volatile int*)&sh.abort) break;
        int g, w;
        stage_gw(i, g, w);
        const int tau = w * kStride32 + lane;
        // lane 0 holds only the left end of lane 1's interval; lanes past step T hold nothing
        const bool dep_lane = lane > 0 && tau <= T;
        const float* st = stages + (size_t)s * SE * kTile;
        using Smp = typename std::conditional<RING, SmpR, SmpF>::type;
        Smp cur[OPW][SE];
        if (TM) {
            // records from tensor memory, in two loads per element pair: the positions
            // (columns 0-7) first; the other groups (columns 8-31) load while the retarded
            // time is solved, and the next pair's positions while this pair's source terms
            // are formed
            const uint32_t tq = sh.tmem + ((uint32_t)(32 * (warp & 3)) << 16);
            uint32_t ra[8], rz[8];
            tmem_ld_x8(tq + tm_col<SE>(s, 0), ra);
            tmem_wait_ld_tie(ra, rz);
#pragma unroll
            for (int jp = 0; jp < SE / 2; ++jp) {
                const uint32_t ta = tq + tm_col<SE>(s, jp);
                uint32_t rc[16], rd[8];
                tmem_ld_x16(ta + 8u, rc);
                tmem_ld_x8(ta + 24u, rd);
                const G2 g0 = g2_of(ra);
                MixedGeom m[OPW];
#pragma unroll
                for (int q = 0; q < OPW; ++q) m[q] = mixed_geom(g0, anc[q], p);
                tmem_wait_ld_tie(rc, rd, m[0].dt, m[0].rx, m[0].ry, m[0].ir);
                if (jp + 1 < SE / 2) tmem_ld_x8(ta + tm_col<SE>(0, 1), ra);
#pragma unroll
                for (int q = 0; q < OPW; ++q)
                    mixed_source<!RING>(m[q], g0, g2_of(rc), g2_of(rc + 8), g2_of(rd), anc[q], p, tau,
                                        cur[q][2 * jp], cur[q][2 * jp + 1]);
                if (jp + 1 < SE / 2) tmem_wait_ld_tie(ra, rz);
            }
        } else {
#pragma unroll
            for (int jp = 0; jp < SE / 2; ++jp) {
                G2 gg[kGroups32];
                const float* tl = st + (size_t)(2 * jp) * kTile + lane * 4;
#pragma unroll
                for (int q = 0; q < kGroups32; ++q) gg[q] = load_g2(tl + q * 2 * kWin * 4);
#pragma unroll
                for (int q = 0; q < OPW; ++q)
                    sample_mixed2<!RING>(gg, anc[q], p, tau, cur[q][2 * jp], cur[q][2 * jp + 1]);
            }
        }
        // the left neighbour: lane l - 1 of the same window (lane 0 receives lane 31's
        // sample and deposits nothing)
        const int rot_src = (lane + 31) & 31;
        int base[OPW];  // ring: tau + ki - 1.5 * 2^23 (deposit_ring)
#pragma unroll
        for (int q = 0; q < OPW; ++q) base[q] = tau + anc[q].ki - kRoundBits;
#pragma unroll
        for (int q = 0; q < OPW; ++q) {
#pragma unroll
            for (int j = 0; j < SE; ++j) {
                const Smp prev = shfl_idx(cur[q][j], rot_src);
                if constexpr (RING)
                    deposit_ring(acc[q], nb, mm, prev, cur[q][j], base[q], ok_obs[q] && dep_lane, bad, more);
                else
                    deposit(acc[q], T, mm, prev, cur[q][j], ok_obs[q] && dep_lane, bad, more);
            }
        }
        // intervals of more than two bins (|Mr| >= 1): their other bins, for the whole warp
        if (__any_sync(0xffffffffu, more)) {
#pragma unroll
            for (int q = 0; q < OPW; ++q) {
#pragma unroll
                for (int j = 0; j < SE; ++j) {
                    const Smp prev = shfl_idx(cur[q][j], rot_src);
                    if constexpr (RING)
                        deposit_rest_ring(acc[q], nb, mm, prev, cur[q][j], base[q], ok_obs[q] && dep_lane, bad);
                    else
                        deposit_rest(acc[q], T, mm, prev, cur[q][j], ok_obs[q] && dep_lane, bad);
                }
            }
            more = false;
        }
        if (RING) {
            // after a window's last group: the 31 bins no later window reaches, and after
            // the last window the rest of the ring
            if (g == ngroups - 1) {
#pragma unroll
                for (int q = 0; q < OPW; ++q) {
                    if (!ok_obs[q]) continue;
                    double* gs = p.acc + (size_t)o[q] * T * 2;
                    ring_flush(acc[q], nb, lo[q] + kStride32 * w, kStride32, gs, T, p.tmod, lane, p.err);
                    if (w == nW - 1) ring_flush(acc[q], nb, lo[q] + kStride32 * nW, nb, gs, T, p.tmod, lane, p.err);
                }
            }
        } else if (w == nW - 1 && (++since_flush == p.flush_groups || g == ngroups - 1)) {
            // FP32 partial sums cover at most `flush_groups` element groups before they are
            // added to the FP64 sums in global memory
#pragma unroll
            for (int q = 0; q < OPW; ++q)
                if (ok_obs[q]) flush_bins(acc[q], p.acc + (size_t)o[q] * T * 2, T, lane, false, p.err);
            since_flush = 0;
        }
        // release the slot; the last warp to finish with it refills it with stage i + NS
        if (TM) tmem_fence_before();
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            if (atomicAdd(&sh.release[s], 1) == nwarps - 1) {
                sh.release[s] = 0;
                if (TM) atomicExch(&sh.claim[s], 0);
                if (i + NS < N) issue(i + NS);
            }
        }
        if (++s == NS) {
            s = 0;
            par ^= 1u;
        }
    }
    // the scratch slot holds whatever the lanes without a bin added; the next item's rows
    // (of another length in a batch) may cover it
    __syncwarp();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < OPW; ++q) acc[q][nb + 1] = make_float2(0.f, 0.f);
    if (__any_sync(0xffffffffu, bad != 0) && lane == 0) flag(p.err, ACUM_DEVERR_ORDER, &p.err->order);
    gbase = g0 + (unsigned)N;
}

template <int SE, int OPW>
__device__ __forceinline__ void mixed_init(unsigned char* smem, size_t stage_off, int NS, MixedShared<SE, OPW>& sh)
{
    constexpr int kTile = kGroups32 * kWin * 4;
    float2* acc_all = reinterpret_cast<float2*>(smem);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + stage_off + (size_t)NS * SE * kTile * sizeof(float));
    for (size_t i = threadIdx.x; i < stage_off / sizeof(float2); i += blockDim.x) acc_all[i] = make_float2(0.f, 0.f);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&bars[s], 1);
            mbar_init(&sh.tfull[s], 1);
            sh.release[s] = 0;
            sh.last[s] = -1;
            sh.claim[s] = 0;
            sh.copied[s] = -1;
        }
        mbar_fence_init();
        sh.abort = 0;
    }
    __syncthreads();
}

// After an abort: wait (bounded) for the copies still in flight before the block exits.
template <int SE, int OPW>
__device__ __forceinline__ void mixed_drain(unsigned char* smem, size_t stage_off, int NS, MixedShared<SE, OPW>& sh)
{
    constexpr int kTile = kGroups32 * kWin * 4;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + stage_off + (size_t)NS * SE * kTile * sizeof(float));
    if (threadIdx.x == 0)
        for (int k = 0; k < NS; ++k) {
            if (sh.last[k] >= 0) (void)mbar_wait_bounded(&bars[k], (uint32_t)(((unsigned)sh.last[k] / NS) & 1u));
            if (sh.copied[k] >= 0)
                (void)mbar_wait_bounded(&sh.tfull[k], (uint32_t)(((unsigned)sh.copied[k] / NS) & 1u));
        }
    __syncthreads();
}

// Single deck: the blocks take the items of a list ordered by observer-tile group, then
// element chunk, then tile within the group, one at a time from a counter in global
// memory.  The blocks running at any time therefore share one or two chunks of records
// in L2 (each record is read from HBM about once per group), and the FP64 sums they add
// into belong to one group of tiles.  When the plan has a ring (p.dual) the ring kernel,
// the wide-ring kernel (if planned) and the whole-row kernel are launched one after the
// other: each tests the records' reach, and all but the first that serves them return at
// once (a ring kernel needs the records to fit its ring, and every kernel leaves them to
// the smaller ring launched before it when they fit that one).
template <int SE, int OPW, bool TM, bool RING>
__global__ void __launch_bounds__(512, 1) tonal_mixed_kernel(const KParams p)
{
    if (p.dual) {
        const float rm = __uint_as_float(*p.rmax);
        const double kb = p.oM / p.dPsi;
        if (RING && !ring_ok(rm, p.vx, p.vy, p.vz, p.a0, kb, p.obs_rmin, p.ring)) return;
        if (p.ring_lo > 0 && ring_ok(rm, p.vx, p.vy, p.vz, p.a0, kb, p.obs_rmin, p.ring_lo)) return;
    }
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ MixedShared<SE, OPW> sh;
    __shared__ int s_item;
    const size_t stage_off = acc_region_bytes(p.W, (RING ? p.ring : p.T) + 2, 8);
    if (TM && threadIdx.x < 32) {  // one block per SM: the allocation does not wait
        tmem_alloc(&sh.tmem, kTmemCols);
        tmem_relinquish();
        tmem_fence_before();
    }
    mixed_init<SE, OPW>(smem, stage_off, p.NS, sh);
    if (TM) tmem_fence_after();
    unsigned gbase = 0;
    const int nitems = p.obs_tiles * p.nchunk;
    const int G = p.tile_group, per_group = G * p.nchunk;
    const int last_g = (p.obs_tiles - 1) / G, last_n = p.obs_tiles - last_g * G;
    for (;;) {
        // items are taken in order from a shared counter, so that the blocks stay within
        // about one item of each other and share one or two chunks of records in L2
        if (threadIdx.x == 0) s_item = atomicAdd(&p.err->item_next, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= nitems) break;
        const int g = item / per_group, r = item - g * per_group;
        const int gn = g == last_g ? last_n : G;
        const int ec = r / gn, ot = g * G + (r - ec * gn);
        const int e0 = ec * p.chunk;
        const int e1 = min(e0 + p.chunk, p.Epad);
        mixed_item<SE, OPW, TM, RING>(p, ot, e0, e1, smem, stage_off, sh, gbase);
        __syncthreads();
        if (sh.abort) {
            mixed_drain<SE, OPW>(smem, stage_off, p.NS, sh);
            break;
        }
    }
    if (TM) {
        tmem_fence_before();
        __syncthreads();
        if (threadIdx.x < 32) tmem_dealloc(sh.tmem, kTmemCols);
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&p.err->item_done, 1) == (int)gridDim.x - 1) {
            atomicExch(&p.err->item_next, 0);
            atomicExch(&p.err->item_done, 0);
        }
    }
}

// Many decks: one block per SM (as many as fit) takes work items from a shared counter
// (largest first, as the host sorts them) until none are left.  Item k is (case,
// observer tile, first element, end element); the case's constants are copied into
// shared memory at the start of each item, and a case whose records fit the bin ring
// (ring > 0 in its constants, decided by the host) runs the ring form, the others whole
// rows.
template <int SE, int OPW>
__global__ void __launch_bounds__(512, 1)
    tonal_batch_kernel(const KParams* __restrict__ cases, const BatchItem* __restrict__ items, int nitems,
                       int* counter, int NS, size_t stage_off)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ MixedShared<SE, OPW> sh;
    __shared__ __align__(16) KParams sp;
    __shared__ BatchItem s_it;
    mixed_init<SE, OPW>(smem, stage_off, NS, sh);
    unsigned gbase = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const int k = atomicAdd(counter, 1);
            s_it = k < nitems ? items[k] : BatchItem{-1, 0, 0, 0};
        }
        __syncthreads();
        const BatchItem it = s_it;
        if (it.c < 0) break;
        constexpr int kWords = (int)(sizeof(KParams) / sizeof(int));
        for (int k = threadIdx.x; k < kWords; k += blockDim.x)
            reinterpret_cast<int*>(&sp)[k] = reinterpret_cast<const int*>(cases + it.c)[k];
        __syncthreads();
        // the item works on a copy, whose constants the compiler keeps in registers instead
        // of reading them from shared memory in the integrand (7334 -> 7173 ms at
        // workload 4; at two observers per warp and 8 elements per stage ptxas keeps a
        // 4-byte spill)
        const KParams lp = sp;
        if (lp.ring > 0)
            mixed_item<SE, OPW, false, true>(lp, it.ot, it.e0, it.e1, smem, stage_off, sh, gbase);
        else
            mixed_item<SE, OPW, false, false>(lp, it.ot, it.e0, it.e1, smem, stage_off, sh, gbase);
        __syncthreads();
        if (sh.abort) {
            mixed_drain<SE, OPW>(smem, stage_off, NS, sh);
            break;
        }
    }
}

constexpr int kMixedSE = 8;   // elements per stage of the whole-row mixed kernel (one observer per warp)
constexpr int kRingSE = 8;    // elements per stage of the ring kernel
constexpr int kRingOPW = 2;   // observers per warp of the ring kernel
// observers per warp of the wide-ring kernels (1024 and 2048 slots): both then run 12 warps
// of 24 and 12 observers (two per warp at 2048 slots would leave 6 warps: 40.3 ms against
// 31.0 ms on 1024 observers of a 4096-step deck; one per warp at 1024 slots 15.1 ms
// against 13.7 ms on a 2048-step deck)
constexpr int kWideOPW[kWideTiers] = {2, 1};
constexpr bool kMixedTmem = false;  // record stages read from tensor memory by default
static_assert(kMaxStages >= 4, "stage bookkeeping");
static_assert(sizeof(SmpF) == 16, "sample record");
constexpr int kSE64 = 2;

// static shared memory of a kernel as compiled (MixedShared<SE> and, in the batched form,
// the case's constants and the current item); an estimate if the query fails
template <typename K>
static size_t static_smem_of(K kernel, size_t estimate)
{
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, kernel) != cudaSuccess) {
        (void)cudaGetLastError();
        return estimate;
    }
    return a.sharedSizeBytes;
}

// static shared memory of the mixed kernels (the ring and whole-row forms of a shape have
// the same)
static size_t mixed_static_smem(int SE, int opw, bool tm)
{
    static size_t v[2][3][9] = {};
    if (SE != 2 && SE != 4 && SE != 8) SE = 8;
    if (opw != 2) opw = 1;
    if (opw == 2) tm = false;
    size_t& x = v[tm ? 1 : 0][opw][SE];
    if (!x) {
        const size_t est = (size_t)1024;
        if (opw == 2)
            x = SE == 2   ? static_smem_of(tonal_mixed_kernel<2, 2, false, true>, est)
                : SE == 4 ? static_smem_of(tonal_mixed_kernel<4, 2, false, true>, est)
                          : static_smem_of(tonal_mixed_kernel<8, 2, false, true>, est);
        else if (tm)
            x = SE == 2   ? static_smem_of(tonal_mixed_kernel<2, 1, true, false>, est)
                : SE == 4 ? static_smem_of(tonal_mixed_kernel<4, 1, true, false>, est)
                          : static_smem_of(tonal_mixed_kernel<8, 1, true, false>, est);
        else
            x = SE == 2   ? static_smem_of(tonal_mixed_kernel<2, 1, false, false>, est)
                : SE == 4 ? static_smem_of(tonal_mixed_kernel<4, 1, false, false>, est)
                          : static_smem_of(tonal_mixed_kernel<8, 1, false, false>, est);
    }
    return x;
}

size_t batch_static_smem(int SE, int opw)
{
    static size_t v[3][9] = {};
    if (SE != 2 && SE != 4 && SE != 8) SE = 8;
    if (opw != 2) opw = 1;
    if (!v[opw][SE]) {
        const size_t est = 1024;
        v[opw][SE] = opw == 2 ? (SE == 2   ? static_smem_of(tonal_batch_kernel<2, 2>, est)
                                 : SE == 4 ? static_smem_of(tonal_batch_kernel<4, 2>, est)
                                           : static_smem_of(tonal_batch_kernel<8, 2>, est))
                              : (SE == 2   ? static_smem_of(tonal_batch_kernel<2, 1>, est)
                                 : SE == 4 ? static_smem_of(tonal_batch_kernel<4, 1>, est)
                                           : static_smem_of(tonal_batch_kernel<8, 1>, est));
    }
    return v[opw][SE];
}

static size_t tonal_smem(int W, int T, int NS, int SE, int real_bytes)
{
    // FP64: double2 per bin; mixed: float2 per bin plus the overflow and scratch slots per row
    const size_t acc = real_bytes == 8 ? acc_region_bytes(W, T, 16) : acc_region_bytes(W, T + 2, 8);
    const int groups = real_bytes == 8 ? kGroups : kGroups32;  // FP64 or FP32 records
    return acc + (size_t)NS * SE * groups * kWin * 4 * real_bytes + (size_t)NS * 8;
}

// One mixed tile: W observers per block (opw per warp), SE elements per stage, rows of
// `ring` slots (0: the T bins of the period); as many stages as the shared memory left
// over holds, and the element chunks of the work items.
static cudaError_t plan_mixed_tile(const TonalRun& r, TonalTile& t, int W_req, int SE_req, int opw, bool tm, int ring,
                                   int items_per_sm, int num_sms, size_t smem_optin)
{
    const int T = r.g.T, rowlen = ring > 0 ? ring : T;
    int SE = (SE_req == 2 || SE_req == 4 || SE_req == 8) ? SE_req : (opw == 2 ? kRingSE : kMixedSE);
    const int NSmin = SE == 8 ? 2 : 4;
    // at most 16 warps (the register limit of 512 threads of 128 registers)
    int W = W_req > 0 ? W_req : 16 * opw;
    W = std::min(W, 16 * opw);
    // keep room in the per-block limit for the kernel's static shared memory
    const size_t budget = smem_optin - mixed_static_smem(SE, opw, tm);
    while (W > opw && tonal_smem(W, rowlen, NSmin, SE, 4) > budget) W -= opw;
    if (tonal_smem(W, rowlen, NSmin, SE, 4) > budget) return cudaErrorInvalidValue;
    if (W_req <= 0) {
        // do not spread few observers over many idle warps
        W = std::max(opw, std::min(W, (r.g.O + opw - 1) / opw * opw));
    }
    W = (W + opw - 1) / opw * opw;
    // as many stages (4..8) as the shared memory left over by the bins holds, without
    // lowering the blocks per SM (registers, ~128 per thread, allow 65536 / (128 * 32 x
    // warps) blocks)
    int NS = NSmin;
    const auto per_sm_at = [&](int ns) { return (int)((228 * 1024) / (tonal_smem(W, rowlen, ns, SE, 4) + 1024)); };
    const int resident = std::max(1, std::min(per_sm_at(NSmin), 65536 / (128 * 32 * (W / opw))));
    while (NS < kMaxStages && tonal_smem(W, rowlen, NS + 1, SE, 4) <= budget && per_sm_at(NS + 1) >= resident) ++NS;
    // tensor-memory form: the stages fit in the block's kTmemCols columns, and one block per
    // SM holds them all
    if (tm) NS = std::max(1, std::min(NS, (int)kTmemCols / (16 * SE)));
    t.W = W;
    t.SE = SE;
    t.NS = NS;
    t.opw = opw;
    t.tm = tm;
    t.ring = ring;
    t.ring_lo = 0;
    t.smem = tonal_smem(W, rowlen, NS, SE, 4);
    // more than half of the shared memory keeps a second block off the SM (a second
    // allocation of the tensor-memory columns would wait for the first block to end)
    if (tm) t.smem = std::max(t.smem, std::min(budget, smem_optin / 2 + 1024));
    const int obs_tiles = (r.g.O + W - 1) / W;
    const int per_sm =
        tm ? 1 : std::max(1, std::min((int)((228 * 1024) / (t.smem + 1024)), 65536 / (128 * 32 * (W / opw))));
    const int slots = num_sms * per_sm;
    // Element chunks whose FP32 records (nW32 x 2048 B per element) take about 32 MB, so
    // that the blocks running at one time (which work on one chunk) find the chunk in L2
    // and each record is read from HBM a few times per launch at most; smaller if needed to
    // give every slot `items_per_sm` items (default 8).  The FP32 bins are added into the
    // FP64 sums within each item (at most 512 elements): larger chunks would re-read
    // records, smaller ones would add FP64 flush traffic.
    const size_t per_elem = (size_t)nwin32(T) * kGroups32 * kWin * 4 * sizeof(float);
    long chunk = (long)std::max<size_t>((size_t)SE, ((size_t)32 << 20) / per_elem);
    chunk = std::min<long>(chunk, 512);
    const int ips = items_per_sm > 0 ? items_per_sm : 8;
    const long want = std::max<long>(1, ((long)ips * slots + obs_tiles - 1) / obs_tiles);
    chunk = std::min(chunk, ((long)r.g.Epad + want - 1) / want);
    chunk = std::max<long>(SE, chunk / SE * SE);
    t.chunk = (int)chunk;
    t.nchunk = (int)(((long)r.g.Epad + chunk - 1) / chunk);
    t.items = obs_tiles * t.nchunk;
    // one group of all observer tiles: grouping them so that their FP64 sums stay in L2
    // re-reads the records once per group and measured no faster
    t.tile_group = obs_tiles;
    t.grid = std::min(t.items, slots);
    t.flush_elems = t.chunk;
    return cudaSuccess;
}

cudaError_t plan_tonal(TonalRun& r, int W_req, int SE_req, int items_per_sm, int num_sms, size_t smem_optin,
                       int opw_req, int tm_req, int rows_only)
{
    const bool f64 = r.precision == ACUM_PLAIN_FP64;
    memset(&r.rows, 0, sizeof(r.rows));
    memset(r.wide, 0, sizeof(r.wide));
    if (!f64) {
        // Mixed: the ring kernel (observers per warp 1 or 2, default 2; elements per stage
        // 2, 4 or 8), with the wide-ring kernels behind it (each in decks of more steps than
        // its slots), and the whole-row kernel (one observer per warp) last, for records
        // that reach too far for every ring; whole rows alone when asked for, with
        // tensor-memory stages, or without the records' reach.
        const bool tm = tm_req == 1 || (tm_req == 0 && kMixedTmem);
        TonalTile rows;
        memset(&rows, 0, sizeof(rows));
        cudaError_t e = plan_mixed_tile(r, rows, std::min(W_req, 16), SE_req, 1, tm, 0, items_per_sm, num_sms,
                                        smem_optin);
        if (e != cudaSuccess) return e;
        if (tm || rows_only || !r.rmax) {
            r.t = rows;
            return cudaSuccess;
        }
        const int opw = opw_req == 1 ? 1 : kRingOPW;
        TonalTile ring;
        memset(&ring, 0, sizeof(ring));
        if (plan_mixed_tile(r, ring, W_req, SE_req, opw, false, kRingSlots, items_per_sm, num_sms, smem_optin) !=
            cudaSuccess) {
            r.t = rows;
            return cudaSuccess;
        }
        ring.ring_lo = 0;
        int below = ring.ring;  // the largest ring planned so far
        for (int k = 0; k < kWideTiers; ++k) {
            if (r.g.T <= kRingSlotsWide[k]) break;
            // a wide ring: as many observers per block as its rows leave room for (one per
            // warp when one is asked for)
            TonalTile wide;
            memset(&wide, 0, sizeof(wide));
            if (plan_mixed_tile(r, wide, W_req, SE_req, opw_req == 1 ? 1 : kWideOPW[k], false, kRingSlotsWide[k],
                                items_per_sm, num_sms, smem_optin) != cudaSuccess)
                break;
            wide.ring_lo = below;
            below = wide.ring;
            r.wide[k] = wide;
        }
        rows.ring_lo = below;
        r.t = ring;
        r.rows = rows;
        return cudaSuccess;
    }
    // FP64: elements per stage 2, one observer per warp
    const int SE = kSE64, opw = 1;
    const int NSmin = 4;
    const int T = r.g.T;
    int W = W_req > 0 ? W_req : 16;
    W = std::min(W, 16);
    const size_t budget = smem_optin - 1024;
    while (W > opw && tonal_smem(W, T, NSmin, SE, 8) > budget) W -= opw;
    if (tonal_smem(W, T, NSmin, SE, 8) > budget) return cudaErrorInvalidValue;
    if (W_req <= 0) W = std::max(1, std::min(W, r.g.O));
    TonalTile& t = r.t;
    t.flush_elems = 1 << 30;
    t.W = W;
    t.SE = SE;
    t.NS = NSmin;
    t.opw = 1;
    t.tm = false;
    t.ring = 0;
    t.ring_lo = 0;
    t.smem = tonal_smem(W, T, NSmin, SE, 8);
    const int obs_tiles = (r.g.O + W - 1) / W;
    // resident blocks per SM: shared memory, and registers (~128 per thread)
    const int per_sm = std::max(1, std::min((int)((228 * 1024) / (t.smem + 1024)), 65536 / (128 * 32 * W)));
    const int slots = num_sms * per_sm;
    const int groups = r.g.Epad / SE;
    const int ips = items_per_sm > 0 ? items_per_sm : 64;
    // number of element chunks among 1 .. ips work items per slot with the smallest
    // wave-quantisation loss (a small charge per extra chunk for its prologue and its
    // flush of the bins); one block per item
    int best = 1;
    double best_cost = 1e30;
    const int maxc = std::max(1, std::min(groups, std::max(1, (ips * slots + obs_tiles - 1) / obs_tiles)));
    for (int c = 1; c <= maxc; ++c) {
        const long items = (long)obs_tiles * c;
        const double waves = (double)items / slots;
        const double eff = waves / std::ceil(waves);
        const double cost = 1.0 / eff + 0.002 * c;
        if (cost < best_cost) {
            best_cost = cost;
            best = c;
        }
    }
    t.nchunk = best;
    const int gpc = (groups + best - 1) / best;
    t.chunk = gpc * SE;
    t.nchunk = (groups + gpc - 1) / gpc;
    t.items = obs_tiles * t.nchunk;
    t.grid = t.items;
    t.tile_group = obs_tiles;
    return cudaSuccess;
}

template <int SE>
static cudaError_t launch_f64_t(const KParams& kp, int items, int threads, size_t smem, cudaStream_t s)
{
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(tonal_f64_kernel<SE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    tonal_f64_kernel<SE><<<items, threads, smem, s>>>(kp);
    return cudaGetLastError();
}

template <int SE, int OPW, bool TM, bool RING>
static cudaError_t launch_mixed_t(const KParams& kp, int grid, int threads, size_t smem, cudaStream_t s)
{
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(tonal_mixed_kernel<SE, OPW, TM, RING>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    tonal_mixed_kernel<SE, OPW, TM, RING><<<grid, threads, smem, s>>>(kp);
    return cudaGetLastError();
}

void fill_kparams(const TonalRun& r, KParams& kp) { fill_kparams(r, r.t, kp); }

void fill_kparams(const TonalRun& r, const TonalTile& tile, KParams& kp)
{
    memset(&kp, 0, sizeof(kp));
    const TonalGeom& g = r.g;
    kp.rec = r.rec;
    kp.Epad = g.Epad;
    kp.T = g.T;
    kp.nW = g.nW;
    kp.nW32 = nwin32(g.T);
    kp.ring = tile.ring;
    kp.ring_lo = tile.ring_lo;
    kp.dual = r.t.ring > 0 ? 1 : 0;
    kp.rmax = r.rmax;
    kp.obs_rmin = g.obs_rmin;
    kp.O = g.O;
    kp.obs32 = r.obs32;
    kp.obs64 = r.obs64;
    const double alpha = g.a0 * g.a0 - (g.vinf[0] * g.vinf[0] + g.vinf[1] * g.vinf[1] + g.vinf[2] * g.vinf[2]);
    kp.a0 = g.a0;
    kp.alpha = alpha;
    kp.ialpha = 1.0 / alpha;
    kp.vx = g.vinf[0];
    kp.vy = g.vinf[1];
    kp.vz = g.vinf[2];
    kp.dTau = g.dTau;
    kp.oM = g.oM;
    kp.dPsi = g.dPsi;
    kp.lpi = g.T * g.dPsi;
    const float a0f = (float)g.a0, alphaf = (float)alpha;
    const float vxf = (float)g.vinf[0], vyf = (float)g.vinf[1], vzf = (float)g.vinf[2];
    const float kbf = (float)(g.oM / g.dPsi);  // bins per second of retarded time
    kp.nalpha2 = make_float2(-alphaf, -alphaf);
    kp.alpha2 = make_float2(alphaf, alphaf);
    kp.nvx2 = make_float2(-vxf, -vxf);
    kp.nvy2 = make_float2(-vyf, -vyf);
    kp.nvz2 = make_float2(-vzf, -vzf);
    kp.a02 = make_float2(a0f, a0f);
    kp.kb2 = make_float2(kbf, kbf);
    kp.tmod = (unsigned)((0x100000000ull + (unsigned long long)g.T - 1) / (unsigned long long)g.T);
    kp.toff = (int)(((1 << 23) + g.T - 1) / g.T * g.T);
    kp.W = tile.W;
    kp.NS = tile.NS;
    kp.chunk = tile.chunk;
    kp.nchunk = tile.nchunk;
    kp.obs_tiles = (g.O + tile.W - 1) / tile.W;
    kp.tile_group = tile.tile_group > 0 ? tile.tile_group : kp.obs_tiles;
    kp.flush_groups = std::max(1, tile.flush_elems / tile.SE);
    kp.acc = r.acc;
    kp.err = r.err;
}

static cudaError_t launch_mixed_tile(const KParams& kp, const TonalTile& t, cudaStream_t s)
{
    const int threads = 32 * (t.W / t.opw);
    if (t.ring > 0) {
        if (t.opw == 2) {
            if (t.SE == 2) return launch_mixed_t<2, 2, false, true>(kp, t.grid, threads, t.smem, s);
            if (t.SE == 4) return launch_mixed_t<4, 2, false, true>(kp, t.grid, threads, t.smem, s);
            return launch_mixed_t<8, 2, false, true>(kp, t.grid, threads, t.smem, s);
        }
        if (t.SE == 2) return launch_mixed_t<2, 1, false, true>(kp, t.grid, threads, t.smem, s);
        if (t.SE == 4) return launch_mixed_t<4, 1, false, true>(kp, t.grid, threads, t.smem, s);
        return launch_mixed_t<8, 1, false, true>(kp, t.grid, threads, t.smem, s);
    }
    if (t.tm) {
        if (t.SE == 2) return launch_mixed_t<2, 1, true, false>(kp, t.grid, threads, t.smem, s);
        if (t.SE == 8) return launch_mixed_t<8, 1, true, false>(kp, t.grid, threads, t.smem, s);
        return launch_mixed_t<4, 1, true, false>(kp, t.grid, threads, t.smem, s);
    }
    if (t.SE == 2) return launch_mixed_t<2, 1, false, false>(kp, t.grid, threads, t.smem, s);
    if (t.SE == 8) return launch_mixed_t<8, 1, false, false>(kp, t.grid, threads, t.smem, s);
    return launch_mixed_t<4, 1, false, false>(kp, t.grid, threads, t.smem, s);
}

cudaError_t launch_tonal(const TonalRun& r, cudaStream_t s)
{
    KParams kp;
    fill_kparams(r, kp);
    if (r.precision == ACUM_PLAIN_FP64) return launch_f64_t<kSE64>(kp, r.t.items, 32 * r.t.W, r.t.smem, s);
    cudaError_t e = launch_mixed_tile(kp, r.t, s);
    if (e != cudaSuccess || r.t.ring == 0) return e;
    // the wide-ring and whole-row kernels behind the ring kernel: each runs when the
    // records reach too far for the rings before it, and returns at once otherwise
    KParams kr;
    for (int k = 0; k < kWideTiers && r.wide[k].ring > 0; ++k) {
        fill_kparams(r, r.wide[k], kr);
        e = launch_mixed_tile(kr, r.wide[k], s);
        if (e != cudaSuccess) return e;
    }
    fill_kparams(r, r.rows, kr);
    return launch_mixed_tile(kr, r.rows, s);
}

size_t batch_smem(int W, int SE, int rowlen)
{
    const int NS = batch_stages(SE);
    return acc_region_bytes(W, rowlen + 2, 8) + (size_t)NS * SE * kGroups32 * kWin * 4 * sizeof(float) +
           (size_t)NS * 8;
}

template <int SE, int OPW>
static int batch_per_sm_t(int W, size_t smem)
{
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tonal_batch_kernel<SE, OPW>, 32 * (W / OPW), smem) !=
            cudaSuccess ||
        per_sm < 1) {
        (void)cudaGetLastError();
        per_sm = 1;
    }
    return per_sm;
}

template <int SE, int OPW>
static cudaError_t launch_batch_t(const KParams* d_cases, const BatchItem* d_items, int nitems, int* d_counter, int W,
                                  int rowlen, int grid, cudaStream_t s)
{
    static size_t configured = 0;
    const size_t smem = batch_smem(W, SE, rowlen);
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(tonal_batch_kernel<SE, OPW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    // as many resident blocks per SM as shared memory and registers allow
    const int per_sm = batch_per_sm_t<SE, OPW>(W, smem);
    tonal_batch_kernel<SE, OPW><<<grid * per_sm, 32 * (W / OPW), smem, s>>>(d_cases, d_items, nitems, d_counter,
                                                                             batch_stages(SE),
                                                                             acc_region_bytes(W, rowlen + 2, 8));
    return cudaGetLastError();
}

int batch_blocks_per_sm(int W, int SE, int opw, int rowlen)
{
    const size_t smem = batch_smem(W, SE, rowlen);
    if (opw == 2)
        return SE == 2 ? batch_per_sm_t<2, 2>(W, smem) : SE == 8 ? batch_per_sm_t<8, 2>(W, smem) : batch_per_sm_t<4, 2>(W, smem);
    return SE == 2 ? batch_per_sm_t<2, 1>(W, smem) : SE == 8 ? batch_per_sm_t<8, 1>(W, smem) : batch_per_sm_t<4, 1>(W, smem);
}

// grid = SMs; the launch puts as many blocks on each SM as fit
cudaError_t launch_tonal_batch(const KParams* d_cases, const BatchItem* d_items, int nitems, int* d_counter, int W,
                               int SE, int opw, int rowlen, int grid, cudaStream_t s)
{
    if (opw != 1 && opw != 2) return cudaErrorInvalidValue;
    if (W < opw || W > 16 * opw || W % opw != 0 || grid < 1) return cudaErrorInvalidValue;
    if (opw == 2) {
        if (SE == 2) return launch_batch_t<2, 2>(d_cases, d_items, nitems, d_counter, W, rowlen, grid, s);
        if (SE == 4) return launch_batch_t<4, 2>(d_cases, d_items, nitems, d_counter, W, rowlen, grid, s);
        if (SE == 8) return launch_batch_t<8, 2>(d_cases, d_items, nitems, d_counter, W, rowlen, grid, s);
        return cudaErrorInvalidValue;
    }
    if (SE == 2) return launch_batch_t<2, 1>(d_cases, d_items, nitems, d_counter, W, rowlen, grid, s);
    if (SE == 4) return launch_batch_t<4, 1>(d_cases, d_items, nitems, d_counter, W, rowlen, grid, s);
    if (SE == 8) return launch_batch_t<8, 1>(d_cases, d_items, nitems, d_counter, W, rowlen, grid, s);
    return cudaErrorInvalidValue;
}

// ------------------------------------------------------------------ finalize

__global__ void finalize_kernel(const double* __restrict__ acc, int O, int T, void* pT, void* pL, void* pA, int mode)
{
    __shared__ double tT[32][33], tL[32][33];
    const int o0 = blockIdx.y * 32, n0 = blockIdx.x * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int o = o0 + k, n = n0 + threadIdx.x;
        double a = 0, b = 0;
        if (o < O && n < T) {
            double2 v = reinterpret_cast<const double2*>(acc)[(size_t)o * T + n];
            a = v.x;
            b = v.y;
        }
        tT[k][threadIdx.x] = a;
        tL[k][threadIdx.x] = b;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int n = n0 + k, o = o0 + threadIdx.x;
        if (n >= T || o >= O) continue;
        const double a = tT[threadIdx.x][k], b = tL[threadIdx.x][k];
        const size_t q = (size_t)n * O + o;
        if (mode == 0) {
            if (pT) reinterpret_cast<double*>(pT)[q] = a;
            if (pL) reinterpret_cast<double*>(pL)[q] = b;
            if (pA) reinterpret_cast<double*>(pA)[q] = a + b;
        } else if (mode == 1) {
            if (pT) reinterpret_cast<double*>(pT)[q] += a;
            if (pL) reinterpret_cast<double*>(pL)[q] += b;
            if (pA) reinterpret_cast<double*>(pA)[q] += a + b;
        } else {
            if (pT) reinterpret_cast<float*>(pT)[q] += (float)a;
            if (pL) reinterpret_cast<float*>(pL)[q] += (float)b;
            if (pA) reinterpret_cast<float*>(pA)[q] += (float)(a + b);
        }
    }
}

cudaError_t launch_finalize(const double* acc, int O, int T, void* pT, void* pL, void* pA, int mode, cudaStream_t s)
{
    dim3 grid((T + 31) / 32, (O + 31) / 32), block(32, 8);
    finalize_kernel<<<grid, block, 0, s>>>(acc, O, T, pT, pL, pA, mode);
    return cudaGetLastError();
}

// One block per 32 x 32 (observer, bin) tile of some case; the case is found by binary
// search over the cases' first tile indices.
__global__ void finalize_batch_kernel(const FinCase* __restrict__ cases, int ncase)
{
    __shared__ double tA[32][33];
    int lo = 0, hi = ncase - 1;
    const int tile = blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cases[mid].tile0 <= tile) lo = mid;
        else hi = mid - 1;
    }
    const FinCase c = cases[lo];
    const int local = tile - c.tile0;
    const int o0 = (local % c.tiles_o) * 32, n0 = (local / c.tiles_o) * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int o = o0 + k, n = n0 + threadIdx.x;
        double a = 0;
        if (o < c.O && n < c.T) {
            const double2 v = reinterpret_cast<const double2*>(c.acc)[(size_t)o * c.T + n];
            a = v.x + v.y;
        }
        tA[k][threadIdx.x] = a;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int n = n0 + k, o = o0 + threadIdx.x;
        if (n < c.T && o < c.O) c.pA[(size_t)n * c.O + o] = tA[threadIdx.x][k];
    }
}

cudaError_t launch_finalize_batch(const FinCase* d_cases, int ncase, int total_tiles, cudaStream_t s)
{
    if (ncase < 1 || total_tiles < 1) return cudaErrorInvalidValue;
    finalize_batch_kernel<<<total_tiles, dim3(32, 8), 0, s>>>(d_cases, ncase);
    return cudaGetLastError();
}

void gauss_taps(double* w)
{
    // mathfunc.cu:350-370 with n_win = 13: sigma = 2, normalised
    const double sd = (13 - 1) / 6.0, amp = 1.0 / (std::sqrt(2.0 * M_PI) * sd);
    double tot = 0.0;
    for (int j = 0; j < 13; ++j) {
        const double x = j - 6;
        w[j] = amp * std::exp(-0.5 * (x * x) / sd / sd);
        tot += w[j];
    }
    for (int j = 0; j < 13; ++j) w[j] = w[j] / tot;
}

}  // namespace acum
