// noalloc.cu -- acum_find_pressure_time_history_noalloc: the reference-shaped tonal
// drop-in for callers that must not allocate device memory.
//
// Who needs it: a solver or plugin host that has handed all device memory to its own pool
// allocator and forbids its components to allocate outside it (a cudaMalloc there fails
// for lack of memory or escapes the host's accounting), and a latency-bound loop that
// cannot afford cudaMalloc/cudaFree, which synchronise the whole device and so stall the
// loop's other streams.  Such a caller still owns and passes its inputs and outputs; what
// the computation needs besides them (the tiled per-step records, the FP64 bin sums and
// the device error word) lives here in one fixed array of device memory that every GPU
// loading this library reserves until process exit.
//
// Limits and behaviour:
//  * the scratch array is kNoAllocBytes = 128 MiB per device; a call whose records
//    (64 bytes per element and record slot: elements rounded up to 8, ceil(nTime / 31)
//    windows of 32 slots) plus FP64 bin sums (16 bytes per observer-step) exceed it is
//    rejected with ACUM_ERR_INVALID and a message that gives both sizes; at most
//    kMaxSurfaces surfaces;
//  * it accepts the inputs the allocating drop-in accepts (nTime >= 4, tObs[t] = t * dPsi
//    within the same tolerance) and refuses the others with the same status;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress)
//    with that device current; make that first call before any stream capture;
//  * every call synchronises `stream` before it returns: it reads E, vInf, tObs and the
//    observers back to the host, and after the kernels the device error word;
//  * every call reuses the same array and leaves its contents behind; the call clears
//    what must start at zero itself, and two calls whose GPU work overlaps (different
//    streams or threads without ordering) race on the array -- serialise them;
//  * no cudaMalloc/cudaFree, no host heap allocation: the small per-surface arrays and
//    tObs (in pieces) are read into fixed stack buffers.
#include <cuda_runtime.h>
#include <stdio.h>
#include <math.h>
#include <string.h>

#include <mutex>

#include "acum_internal.h"
#include "ctx.h"

namespace acum {

constexpr size_t kNoAllocBytes = 128ull << 20;
constexpr int kMaxSurfaces = 256;
constexpr int kMaxDevices = 64;

// the scratch: tiled records first, then the [obs][step][2] FP64 bin sums
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

static std::mutex g_na_mu;
static void* g_na_ptr[kMaxDevices];
// the last message of this thread (no lock, no heap)
static thread_local char g_na_msg[256];
constexpr int kTobsPiece = 1024;  // tObs is checked in pieces of this many steps

// Records straight from the reference's AoS arrays; the element's surface and offsets
// are found from E[] and the X/N/V/PR pointer arrays on the device (no host tables).
__global__ void noalloc_records_kernel(const float* __restrict__ X, const float* __restrict__ N,
                                       const float* __restrict__ V, const float* __restrict__ PR,
                                       const int* __restrict__ E, const int* __restrict__ XPtr,
                                       const int* __restrict__ NPtr, const int* __restrict__ VPtr,
                                       const int* __restrict__ PRPtr, int nSurf, int Etot, int T, int nW32, double a0,
                                       double rho, double vx_inf, double vy_inf, double vz_inf,
                                       float* __restrict__ rec, unsigned* rmax)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Etot * T) return;
    const int e = (int)(idx / T), t = (int)(idx % T);
    int s = 0, base = 0;
    while (s < nSurf - 1 && e >= base + E[s]) {
        base += E[s];
        ++s;
    }
    const int j = e - base;
    const float* x = X + XPtr[s] + (size_t)j * T * 4 + (size_t)t * 4;
    const float* n = N + NPtr[s] + (size_t)j * T * 6 + (size_t)t * 6;
    const float* v = V + VPtr[s] + (size_t)j * T * 6 + (size_t)t * 6;
    const float* pr = PR + PRPtr[s] + (size_t)j * T * 2 + (size_t)t * 2;
    const double D1 = 1.0 / (4.0 * M_PI * a0), ia0 = 1.0 / a0;
    const double vx = v[0], vy = v[1], vz = v[2], nx = n[0], ny = n[1], nz = n[2], P = pr[0], Pd = pr[1];
    const double ds = x[3];
    const double L[3] = {P * nx, P * ny, P * nz};
    double r[20];
    r[0] = x[0]; r[1] = x[1]; r[2] = x[2]; r[3] = D1 * ds;
    r[4] = vx * ia0; r[5] = vy * ia0; r[6] = vz * ia0; r[7] = (vx * vx + vy * vy + vz * vz) * ia0 * ia0;
    r[8] = (double)v[3] * ia0; r[9] = (double)v[4] * ia0; r[10] = (double)v[5] * ia0;
    r[11] = D1 * rho * (vx * nx + vy * ny + vz * nz) * a0 * ds;
    r[12] = L[0]; r[13] = L[1]; r[14] = L[2]; r[15] = (L[0] * vx + L[1] * vy + L[2] * vz) * ia0;
    r[16] = Pd * nx + P * (double)n[3]; r[17] = Pd * ny + P * (double)n[4]; r[18] = Pd * nz + P * (double)n[5];
    r[19] = (double)x[0] * vx_inf + (double)x[1] * vy_inf + (double)x[2] * vz_inf;
    float f32[16];
    rec32_fields<double>(r, r[3], r[11], r + 4, r + 8, r + 12, r + 16, f32);
    rec32_store(rec, e, nW32, T, t, f32);
    note_radius(rmax, sqrtf(f32[0] * f32[0] + f32[1] * f32[1] + f32[2] * f32[2]));
}

}  // namespace acum

using namespace acum;

extern "C" const char* acum_noalloc_last_error(void) { return g_na_msg; }

extern "C" int acum_find_pressure_time_history_noalloc(const float* rObs, const float* tObs, float* pT, float* pL,
                                                       float* pA, const float* Xham, const float* Nham,
                                                       const float* Vham, const float* PRham, int nSurf,
                                                       const int* XPtr, const int* NPtr, const int* VPtr,
                                                       const int* PRPtr, const int* E, int nObs, int nTime,
                                                       float dPsi, float dTau, float a0, float rhoRef,
                                                       const float* vInf, float oM, void* stream)
{
    acum::NvtxRange nvtx_range_("acum_find_pressure_time_history_noalloc");
    auto bad = [](int code, const char* m) {
        snprintf(g_na_msg, sizeof g_na_msg, "%s", m);
        return code;
    };
    if (!rObs || !tObs || !pT || !pL || !pA || !Xham || !Nham || !Vham || !PRham || !XPtr || !NPtr || !VPtr ||
        !PRPtr || !E || !vInf)
        return bad(ACUM_ERR_INVALID, "findPressureTimeHistory_noalloc: null argument");
    if (nSurf <= 0 || nSurf > kMaxSurfaces || nObs <= 0 || nTime < 4)
        return bad(ACUM_ERR_INVALID, "findPressureTimeHistory_noalloc: sizes (1..256 surfaces, nTime >= 4)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: no current device");
    void* scratch = nullptr;
    {
        // set-up once per device, with that device current
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_ptr[dev]) {
            cudaError_t e = cudaGetSymbolAddress(&g_na_ptr[dev], g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_na_ptr[dev] = nullptr;
                snprintf(g_na_msg, sizeof g_na_msg, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
                return ACUM_ERR_CUDA;
            }
        }
        scratch = g_na_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    int hE[kMaxSurfaces];
    float hv[3];
    if (cudaMemcpyAsync(hE, E, nSurf * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(hv, vInf, 3 * sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: reading E/vInf failed");
    // the kernel bins on the uniform grid main.cu:124 builds; refuse another tObs, with the
    // tolerance of the allocating drop-in
    for (int t0 = 0; t0 < nTime; t0 += kTobsPiece) {
        float ht[kTobsPiece];
        const int n = nTime - t0 < kTobsPiece ? nTime - t0 : kTobsPiece;
        if (cudaMemcpyAsync(ht, tObs + t0, n * sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: reading tObs failed");
        for (int k = 0; k < n; ++k) {
            const int t = t0 + k;
            const double want = (double)(float)(t * dPsi);
            if (fabs((double)ht[k] - want) > 1e-6 * fabs((double)dPsi) * (1 + t))
                return bad(ACUM_ERR_UNSUPPORTED, "findPressureTimeHistory_noalloc: tObs must be t*dPsi");
        }
    }
    // the observers' smallest distance from the origin (the mixed ring kernel's test),
    // read in pieces
    double obs_rmin = 1.0e300;
    for (int o0 = 0; o0 < nObs; o0 += kTobsPiece / 3) {
        float ho[kTobsPiece];
        const int n = nObs - o0 < kTobsPiece / 3 ? nObs - o0 : kTobsPiece / 3;
        if (cudaMemcpyAsync(ho, rObs + 3 * (size_t)o0, 3 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: reading rObs failed");
        const double m = obs_min_distance(ho, n);
        if (!(m >= obs_rmin)) obs_rmin = m;
    }
    long long Et = 0;
    for (int i = 0; i < nSurf; ++i) {
        if (hE[i] < 0) return bad(ACUM_ERR_INVALID, "findPressureTimeHistory_noalloc: negative element count");
        Et += hE[i];
    }
    if (Et <= 0) return bad(ACUM_ERR_INVALID, "findPressureTimeHistory_noalloc: no elements");
    const int nW = (nTime + kWin - 1) / kWin, nW32 = nwin32(nTime);
    const long long Epad = (Et + 7) / 8 * 8;
    const size_t rec_bytes = (size_t)Epad * nW32 * kGroups32 * kWin * 4 * sizeof(float);
    const size_t acc_off = (rec_bytes + 255) / 256 * 256;
    const size_t acc_bytes = (size_t)nObs * nTime * 2 * sizeof(double);
    if (acc_off + acc_bytes > kNoAllocBytes) {
        snprintf(g_na_msg, sizeof g_na_msg,
                 "findPressureTimeHistory_noalloc: needs %zu bytes of scratch (records %zu + sums %zu), the "
                 "maximum is %zu",
                 acc_off + acc_bytes, rec_bytes, acc_bytes, kNoAllocBytes);
        return ACUM_ERR_INVALID;
    }
    float* rec = reinterpret_cast<float*>(scratch);
    double* acc = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(scratch) + acc_off);
    // the device error word and the records' largest |x| live in the scratch too (after
    // the sums)
    const size_t err_off = (acc_off + acc_bytes + 255) / 256 * 256;
    const size_t err_bytes = (sizeof(DeviceErr) + 15) / 16 * 16 + 16;
    if (err_off + err_bytes > kNoAllocBytes)
        return bad(ACUM_ERR_INVALID, "findPressureTimeHistory_noalloc: no room for the error word");
    DeviceErr* derr = reinterpret_cast<DeviceErr*>(reinterpret_cast<unsigned char*>(scratch) + err_off);
    unsigned* rmax = reinterpret_cast<unsigned*>(reinterpret_cast<unsigned char*>(derr) + err_bytes - 16);
    // the array keeps the previous call's contents: clear the record padding, the sums,
    // the error word and the radius
    if (cudaMemsetAsync(rec, 0, rec_bytes, st) != cudaSuccess || cudaMemsetAsync(acc, 0, acc_bytes, st) != cudaSuccess ||
        cudaMemsetAsync(derr, 0, err_bytes, st) != cudaSuccess)
        return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: clearing scratch failed");
    const long long n = Et * nTime;
    noalloc_records_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(Xham, Nham, Vham, PRham, E, XPtr, NPtr, VPtr,
                                                                   PRPtr, nSurf, (int)Et, nTime, nW32, a0, rhoRef,
                                                                   (double)hv[0], (double)hv[1], (double)hv[2], rec,
                                                                   rmax);
    if (cudaGetLastError() != cudaSuccess)
        return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: launch of the records kernel failed");
    int sms = 0, optin = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    TonalRun r;
    memset(&r, 0, sizeof(r));
    r.g.E = (int)Et;
    r.g.Epad = (int)Epad;
    r.g.T = nTime;
    r.g.nW = nW;
    r.g.O = nObs;
    r.g.a0 = a0;
    r.g.rho = rhoRef;
    r.g.oM = oM;
    r.g.dPsi = dPsi;
    r.g.dTau = dTau;
    r.g.lpi = nTime * (double)dPsi;
    for (int q = 0; q < 3; ++q) r.g.vinf[q] = hv[q];
    r.g.obs_rmin = obs_rmin;
    r.precision = ACUM_MIXED;
    if (plan_tonal(r, 0, 0, 0, sms, (size_t)optin) != cudaSuccess)
        return bad(ACUM_ERR_UNSUPPORTED, "findPressureTimeHistory_noalloc: no tile shape fits this nTime");
    r.rec = rec;
    r.rmax = rmax;
    r.obs32 = rObs;
    r.obs64 = nullptr;
    r.acc = acc;
    r.err = derr;
    if (launch_tonal(r, st) != cudaSuccess || launch_finalize(acc, nObs, nTime, pT, pL, pA, 2, st) != cudaSuccess)
        return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: launch failed");
    DeviceErr h;
    if (cudaMemcpyAsync(&h, r.err, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return bad(ACUM_ERR_CUDA, "findPressureTimeHistory_noalloc: kernel failed");
    if (h.bits & ACUM_DEVERR_TIMEOUT) return bad(ACUM_ERR_TIMEOUT, "a bounded shared-memory pipeline wait ran out");
    return ACUM_OK;
}
