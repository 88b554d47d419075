// Permeable-surface preprocessing on the GPU: preprocess_per (preprocess.cu:8-226).
//
//  per_prep_kernel   one block per element; the element's series are read from the
//                    reference's AoS arrays (variables.cu:11-42 field order, nPRham = 4
//                    as main.cu:87 sets it for permeable decks) and written back in place.
//
// The arithmetic is FP64 whatever the storage type, and follows the reference's order of
// operations with no fused multiply-adds (explicit __dmul_rn / __dadd_rn where the
// compiler would contract), so that with double storage the outputs equal the
// reference's FP64 build bit for bit, and with float storage they are those FP64 results
// rounded once.  The reference's FP32 build rounds every intermediate to float instead.
// The kernel is bound by the FP64 pipe: the quotients by 2 dTau are formed from its
// reciprocal with FMA corrections that give the IEEE quotient (div_by), and the median's
// comparisons run on integer keys.
//
// Work per element: five flow series (rho, u, v, w, P) scaled, optionally filtered (two
// passes of a 3-point periodic median and a 13-tap periodic Gaussian, preprocess.cu:
// 113-137) and differentiated (periodic or end-biased central differences, preprocess.cu:
// 150-163); the normal's periodic derivative (166-168); the position scaled, its
// derivative V and V's derivative (172-180).  Each series goes through two FP64 rows in
// shared memory, one at a time, so 16 bytes per step suffice (64 KB at 4096 steps).
#include "acum_internal.h"

namespace acum {

namespace {

constexpr int kPerThreads = 256;

template <typename S>
struct PerPtrs {
    S* X;   // [..][T][4]  x, y, z, ds
    S* N;   // [..][T][6]  n, ndot
    S* V;   // [..][T][6]  V, Vdot
    S* U;   // [..][T][6]  u, udot
    S* PR;  // [..][T][4]  P, Pdot, rho, rhodot
};

// Correctly rounded a / b from y = RN(1/b) with FMA corrections: Markstein's theorem
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990; Cornea-Hasegan, Golliver & Markstein,
// ARITH-14, 1999, Theorem 1): if y = RN(1/b) and q is within 1 ulp of a/b, then
// r = a - b q is exact and RN(q + r y) = RN(a/b).  q = RN(a y) followed by one correction
// is within 1 ulp; the second correction then gives the IEEE quotient, for a/b in the
// normal range.  A zero numerator keeps its sign through the product a y.  Five FP64
// operations instead of a full division (the FP64 pipe bounds this kernel).
__device__ __forceinline__ double div_by(double a, double b, double y)
{
    double q = __dmul_rn(a, y);
    double r = __fma_rn(-q, b, a);
    q = __fma_rn(r, y, q);
    r = __fma_rn(-q, b, a);
    q = __fma_rn(r, y, q);
    return a == 0.0 ? __dmul_rn(a, y) : q;
}

// central difference with the reference's division (mathfunc.cu:132-140);
// y = RN(1 / two_dt)
__device__ __forceinline__ double cdiff(double up, double um, double two_dt, double y)
{
    return div_by(up - um, two_dt, y);
}

// A key whose signed-integer order is the order of the (non-NaN) doubles, -0 and +0
// equal: the median's comparisons run on the integer pipe instead of the FP64 pipe.
__device__ __forceinline__ long long order_key(double v)
{
    long long b = __double_as_longlong(v);
    b = b == (long long)0x8000000000000000ULL ? 0LL : b;
    return b < 0 ? (b ^ 0x7FFFFFFFFFFFFFFFLL) : b;
}

// d/dtau of the series in row `src` at step t: periodic, or the end-biased form
// (mathfunc.cu:142-159: central interior, ends from 3 du[1] - 3 du[2] + du[3])
__device__ __forceinline__ double series_deriv(const double* src, int t, int T, double two_dt, double y, bool biased)
{
    if (!biased || (t > 0 && t < T - 1)) {
        const int tm = t == 0 ? T - 1 : t - 1, tp = t == T - 1 ? 0 : t + 1;
        return cdiff(src[tp], src[tm], two_dt, y);
    }
    const int s = t == 0 ? 1 : -1;
    const int k1 = t + s, k2 = t + 2 * s, k3 = t + 3 * s;
    const double d1 = cdiff(src[k1 + 1], src[k1 - 1], two_dt, y);
    const double d2 = cdiff(src[k2 + 1], src[k2 - 1], two_dt, y);
    const double d3 = cdiff(src[k3 + 1], src[k3 - 1], two_dt, y);
    return __dadd_rn(__dsub_rn(__dmul_rn(3.0, d1), __dmul_rn(3.0, d2)), d3);
}

// Outputs of the 13-tap Gaussian per thread.  The taps are symmetric and bit-identical in
// pairs (w[k] = w[12 - k]: gauss_taps forms both from the same (k - 6)^2), so the product
// w[k] Q[q] of output t is also the product w[12 - k] Q[q] of output t + 2k - 12; within a
// run of consecutive outputs each product is formed once (7 + 42 / kGaussRun per output
// instead of 13), while every output still adds its 13 products in the reference's order.
constexpr int kGaussRun = 16;

// two passes of (3-point periodic median, 13-tap periodic Gaussian) on row P, Q scratch
// (mathfunc.cu:208-341 and 375-421); T >= 6, so that one wrap brings every tap of an
// output into the period
__device__ void lowpass_rows(double* P, double* Q, int T, const double* w)
{
    double wr[7];  // the distinct taps, in registers: their products then repeat exactly
#pragma unroll
    for (int j = 0; j < 7; ++j) wr[j] = w[j];
    for (int pass = 0; pass < 2; ++pass) {
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            const double l = P[t == 0 ? T - 1 : t - 1], m = P[t], r = P[t == T - 1 ? 0 : t + 1];
            const long long kl = order_key(l), km = order_key(m), kr = order_key(r);
            const long long hi = max(max(kl, km), kr), lo = min(min(kl, km), kr);
            Q[t] = (kl < hi && kl > lo) ? l : ((km < hi && km > lo) ? m : r);
        }
        __syncthreads();
        const int nruns = (T + kGaussRun - 1) / kGaussRun;
        for (int r = threadIdx.x; r < nruns; r += blockDim.x) {
            const int t0 = r * kGaussRun;
            // qw[i] = Q[t0 - 6 + i] (periodic); the loads past one wrap feed only outputs
            // past the period's end, which are not stored
            double qw[kGaussRun + 12];
#pragma unroll
            for (int i = 0; i < kGaussRun + 12; ++i) {
                int q = t0 - 6 + i;
                q = q < 0 ? q + T : (q > T - 1 ? q - T : q);
                qw[i] = Q[min(q, T - 1)];
            }
#pragma unroll
            for (int s = 0; s < kGaussRun; ++s) {
                double acc = 0.0;
#pragma unroll
                for (int k = 0; k < 13; ++k) acc = __dadd_rn(acc, __dmul_rn(wr[k < 6 ? k : 12 - k], qw[s + k]));
                if (t0 + s < T) P[t0 + s] = acc;
            }
        }
        __syncthreads();
    }
}

template <typename S>
__global__ void __launch_bounds__(kPerThreads) per_prep_kernel(PerPtrs<S> p, PerArgs a)
{
    extern __shared__ __align__(16) unsigned char sm[];
    const int T = a.T;
    double* P = reinterpret_cast<double*>(sm);  // [T]
    double* Q = P + T;                           // [T]
    const int e = blockIdx.x;
    S* X = p.X + a.xoff[e];
    S* N = p.N + a.noff[e];
    S* V = p.V + a.voff[e];
    S* U = p.U + a.uoff[e];
    S* PR = p.PR + a.proff[e];
    const double two_dt = a.two_dt, y = a.inv_two_dt;
    const bool biased = a.periodic != 1;

    // flow series: rho (PR 2), u (U 0..2), P (PR 0), in the reference's order v1..v5
    for (int v = 0; v < 5; ++v) {
        S* col = v == 0 ? PR + 2 : (v == 4 ? PR : U + (v - 1));
        const int stride = v == 0 || v == 4 ? 4 : 6;
        S* dcol = v == 0 ? PR + 3 : (v == 4 ? PR + 1 : U + (v + 2));
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            const double raw = (double)col[(size_t)t * stride];
            double s;
            if (v == 0) s = raw * a.rhoRef;
            else if (v == 4) s = raw * 0.5 * a.rhoRef * a.mref2 * a.a02;  // left to right (preprocess.cu:66)
            else s = raw * a.a0;
            P[t] = s;
        }
        __syncthreads();
        if (a.lowpass == 1) lowpass_rows(P, Q, T, a.gauss);
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            col[(size_t)t * stride] = (S)P[t];
            dcol[(size_t)t * stride] = (S)series_deriv(P, t, T, two_dt, y, biased);
        }
        __syncthreads();
    }
    // normal: periodic derivative of the unchanged n (preprocess.cu:166-168)
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const int tm = t == 0 ? T - 1 : t - 1, tp = t == T - 1 ? 0 : t + 1;
        for (int c = 0; c < 3; ++c)
            N[(size_t)t * 6 + 3 + c] =
                (S)cdiff((double)N[(size_t)tp * 6 + c], (double)N[(size_t)tm * 6 + c], two_dt, y);
        // panel area (preprocess.cu:56): (ds CFDscale) CFDscale
        X[(size_t)t * 4 + 3] = (S)((double)X[(size_t)t * 4 + 3] * a.cfd * a.cfd);
    }
    // position: scaled x, V = dx/dtau, Vdot = dV/dtau, both periodic (preprocess.cu:172-180)
    for (int c = 0; c < 3; ++c) {
        for (int t = threadIdx.x; t < T; t += blockDim.x) P[t] = (double)X[(size_t)t * 4 + c] * a.cfd;
        __syncthreads();
        for (int t = threadIdx.x; t < T; t += blockDim.x) Q[t] = series_deriv(P, t, T, two_dt, y, false);
        __syncthreads();
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            X[(size_t)t * 4 + c] = (S)P[t];
            V[(size_t)t * 6 + c] = (S)Q[t];
            V[(size_t)t * 6 + 3 + c] = (S)series_deriv(Q, t, T, two_dt, y, false);
        }
        __syncthreads();
    }
}

template <typename S>
cudaError_t launch_per_t(S* X, S* N, S* V, S* U, S* PR, const PerArgs& a, cudaStream_t s)
{
    const size_t smem = (size_t)a.T * 2 * sizeof(double);
    if (smem > 48 * 1024) {
        cudaError_t err =
            cudaFuncSetAttribute(per_prep_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    PerPtrs<S> p{X, N, V, U, PR};
    per_prep_kernel<S><<<a.E, kPerThreads, smem, s>>>(p, a);
    return cudaGetLastError();
}

// The rows of a permeable deck as read_surf leaves them (io.cu:263-293): each 12-column
// row x y z u v w P rho ds nx ny nz goes to Xham (x, y, z, ds), Nham (n), Uham (u) and
// PRham (P at 0, rho at 2); the derivative columns and Vham start at zero and are all
// written by the preprocessing.  One thread per (element, step); FP64 storage.
__global__ void per_rows_kernel(const float* __restrict__ raw, const long long* __restrict__ raw_off,
                                const int* __restrict__ e_surf, const int* __restrict__ e_local,
                                const int* __restrict__ e_count, int E, int T, double* X, double* N, double* V,
                                double* U, double* PR)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)E * T) return;
    const int e = (int)(idx / T), t = (int)(idx % T);
    const int s = e_surf[e];
    const float* r = raw + raw_off[s] + ((size_t)t * e_count[s] + e_local[e]) * 12;
    const size_t k = (size_t)e * T + t;
    double* x = X + k * 4;
    double* n = N + k * 6;
    double* v = V + k * 6;
    double* u = U + k * 6;
    double* pr = PR + k * 4;
    x[0] = r[0]; x[1] = r[1]; x[2] = r[2]; x[3] = r[8];
    u[0] = r[3]; u[1] = r[4]; u[2] = r[5]; u[3] = 0.0; u[4] = 0.0; u[5] = 0.0;
    pr[0] = r[6]; pr[1] = 0.0; pr[2] = r[7]; pr[3] = 0.0;
    n[0] = r[9]; n[1] = r[10]; n[2] = r[11]; n[3] = 0.0; n[4] = 0.0; n[5] = 0.0;
    for (int c = 0; c < 6; ++c) v[c] = 0.0;
}

}  // namespace

cudaError_t launch_per_rows(const float* raw, const long long* raw_off, const int* e_surf, const int* e_local,
                            const int* e_count, int E, int T, double* const d[5], cudaStream_t s)
{
    const long long n = (long long)E * T;
    if (n <= 0) return cudaErrorInvalidValue;
    per_rows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(raw, raw_off, e_surf, e_local, e_count, E, T, d[0],
                                                               d[1], d[2], d[3], d[4]);
    return cudaGetLastError();
}

cudaError_t launch_per_prep(void* X, void* N, void* V, void* U, void* PR, bool is_double, const PerArgs& a,
                            cudaStream_t s)
{
    if (a.E < 1 || a.T < 4 || a.T > kMaxPerSteps) return cudaErrorInvalidValue;
    if (is_double)
        return launch_per_t<double>((double*)X, (double*)N, (double*)V, (double*)U, (double*)PR, a, s);
    return launch_per_t<float>((float*)X, (float*)N, (float*)V, (float*)U, (float*)PR, a, s);
}

}  // namespace acum
