// acum_internal.h -- declarations shared by the CUDA translation units and the C++ host
// layer of libacum.  Not part of the public ABI (include/acum.h).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/acum.h"

namespace acum {

// Record layout of one element-step for the tonal kernels.
// FP64 records (the plain form and the adjoints): 5 groups of 4 reals, a lane reads its
// step with 2x128-bit loads per group.
//   g0: x, y, z, dsD          (dsD   = D1 * ds,              D1 = 1/(4 pi a0))
//   g1: Mx, My, Mz, M2        (M     = V / a0,  M2 = |V|^2 / a0^2)
//   g2: Mdx, Mdy, Mdz, ATD    (Md    = Vdot / a0, ATD = D1 * rho0 * (V.n) * a0 * ds)
//   g3: Lx, Ly, Lz, Lm        (L     = P n,  Lm = L.V / a0)
//   g4: Ldx, Ldy, Ldz, xv     (Ldot  = Pdot n + P ndot, xv = x.vInf)
// FP32 records (the mixed form): the 16 fields the integrand cannot do without, 4 groups
// of 4 floats, so that a lane reads an element pair's step with 8 128-bit loads; the
// panel weight dsD is folded into the loading vectors, and |M|^2, L.M and x.vInf are
// recomputed from the fields they are made of:
//   g0: x, y, z, ATD
//   g1: Mx, My, Mz, Ldx'      (Ld' = dsD Ldot)
//   g2: Mdx, Mdy, Mdz, Ldy'
//   g3: Lx', Ly', Lz', Ldz'   (L'  = dsD L)
// In HBM the FP64 records are tiled [element][window][group][32 steps][4]: an (element,
// 32-step window) tile is contiguous (5120 B), which is what one bulk (TMA) copy moves
// into shared memory.  The FP32 records interleave pairs of elements so that the mixed
// kernel reads the two elements' values of a field as one register pair (the operand of
// a packed FP32 instruction): [element pair][window][group][half][32 lanes][4], half 0 =
// (f0 of e, f0 of e+1, f1 of e, f1 of e+1), half 1 = the same for fields 2 and 3; an
// (element pair, window) tile is 4096 B.  Their windows overlap: window w, lane l holds
// step (31 w + l) mod T for 31 w + l = 0 .. T (lanes past T hold zeros), so lane l - 1
// of the same window holds the left end of lane l's source interval and the last window
// reaches step T, which is step 0 one period on (the periodic wrap of core.cu:173-194).
// ceil(T / 31) windows.
constexpr int kGroups = 5;    // FP64 records
constexpr int kGroups32 = 4;  // FP32 records
constexpr int kWin = 32;
constexpr int kStride32 = 31;  // steps between the FP32 records' windows
constexpr int kFields = 18;  // x,y,z,ds, n(3), ndot(3), V(3), Vdot(3), P, Pdot

__host__ __device__ __forceinline__ int nwin32(int T) { return (T + kStride32 - 1) / kStride32; }

// float offset of field c (0..3) of group q (0..3) of element e at lane `lane` of window
// w of the FP32 records
__host__ __device__ __forceinline__ size_t rec32_offset(int e, int nW32, int w, int lane, int q, int c)
{
    return ((((size_t)(e >> 1) * nW32 + w) * kGroups32 + q) * 2 + (c >> 1)) * (kWin * 4) + (size_t)lane * 4 +
           (size_t)((c & 1) * 2 + (e & 1));
}

// Stores the 16 FP32 fields f of element e at step t into every slot of the FP32 records
// that holds that step: lane t mod 31 of window t / 31, also lane 31 of the window before
// when t is a multiple of 31, and for t = 0 also the slot of step T.
__host__ __device__ __forceinline__ void rec32_store(float* rec, int e, int nW32, int T, int t, const float* f)
{
    for (int k = 0; k < 2; ++k) {
        if (k == 1 && t != 0) break;
        const int tau = k == 0 ? t : T;
        const int w = tau / kStride32, l = tau - w * kStride32;
        for (int a = 0; a < 2; ++a) {
            const int ww = a == 0 ? w : w - 1, ll = a == 0 ? l : kStride32;
            if (a == 1 && (l != 0 || w == 0)) break;
            if (ww >= nW32) continue;
            for (int q = 0; q < kGroups32; ++q)
                for (int c = 0; c < 4; ++c) rec[rec32_offset(e, nW32, ww, ll, q, c)] = f[4 * q + c];
        }
    }
}

// Mixed ring form: a bound, in observer-time bins and with a margin, on how far a
// sample's observer time lies from its step plus the observer's anchor (the retarded
// time of the origin): |t - t0| <= |x| / (a0 - |vInf|), because the travel time through a
// uniformly moving medium changes by at most 1 / (a0 - |vInf|) per unit of source
// displacement; r = the records' largest |x|, kb = oM / dPsi bins per second.  1e30 when
// r is not finite or the flight is not subsonic.
__host__ __device__ __forceinline__ double ring_reach_bins(float r, double vx, double vy, double vz, double a0,
                                                           double kb)
{
    const double vm = sqrt(vx * vx + vy * vy + vz * vz);
    if (!(r <= 1.0e30f) || !(vm < 0.999 * a0)) return 1.0e30;
    return (double)r * kb / (a0 - vm) * 1.0001 + 2.0;
}
// Whether the ring kernel serves a deck: a ring of R slots holds every bin a window of 31
// intervals can reach, and the observer-time offset of every sample is bounded by the
// reach, so that the ring kernel needs no per-sample range check.  The second holds when
// the term b = alpha t0 + D0.v + (D0 - x).v of the retarded-time difference quadratic
// stays positive for every source point x and observer D0 (then its denominator b +
// sqrt(q) >= b > 0 and |dt| keeps its bound |x| / (a0 - |vInf|)): b >= sqrt(alpha)
// |D0| - |x| |vInf|, so it suffices that sqrt(alpha) min|D0| > 1.01 |x|max |vInf|; with no
// flight b = alpha t0 >= 0 and a zero b comes with a non-negative discriminant term.
// obs_rmin = the smallest observer distance from the origin (< 0: unknown).
__host__ __device__ __forceinline__ bool ring_ok(float r, double vx, double vy, double vz, double a0, double kb,
                                                 double obs_rmin, int R)
{
    const double reach = ring_reach_bins(r, vx, vy, vz, a0, kb);
    if (!(2.0 * reach + 40.0 <= (double)R)) return false;
    const double vm = sqrt(vx * vx + vy * vy + vz * vz);
    if (vm == 0.0) return true;
    return obs_rmin >= 0.0 && sqrt(a0 * a0 - vm * vm) * obs_rmin > 1.01 * (double)r * vm;
}

// the smallest distance from the origin of n observers given as FP32 (x, y, z) triples
inline double obs_min_distance(const float* xyz, long long n)
{
    double m = n > 0 ? 1.0e300 : -1.0;
    for (long long i = 0; i < n; ++i) {
        const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        const double d = sqrt(x * x + y * y + z * z);
        if (!(d >= m)) m = d;  // a NaN distance makes the minimum NaN (unknown)
    }
    return m;
}

#ifdef __CUDACC__
// The largest source distance from the origin |x| among the records a kernel writes, as
// the bits of a non-negative float in *word (unsigned order = float order; a NaN
// distance is above every finite one): a warp-wide maximum, then one atomic per warp.
// Every lane of the warp that is still running calls it.
__device__ __forceinline__ void note_radius(unsigned* word, float r)
{
    if (!word) return;
    const unsigned mask = __activemask();
    const unsigned m = __reduce_max_sync(mask, __float_as_uint(fabsf(r)));
    if ((threadIdx.x & 31) == (unsigned)(__ffs(mask) - 1)) atomicMax(word, m);
}
#endif

struct DeviceErr {
    unsigned int bits;
    unsigned int disc, order, nonfinite, timeout;
    // work-list counters of the persistent tonal kernel: the next item to take and the
    // blocks done; the last block of a launch sets both back to zero
    int item_next, item_done;
};

struct TonalGeom {
    int E, Epad, T, nW, O;
    double a0, rho, oM, dPsi, dTau, lpi;  // dPsi in radians
    double vinf[3];
    double obs_rmin;  // smallest observer distance from the origin (of the FP32 positions; < 0 unknown)
};

struct TonalTile {
    int W;      // observers (warps) per block
    int SE;     // elements per pipeline stage
    int NS;     // pipeline stages
    int chunk;  // elements per work item (multiple of SE)
    int nchunk;
    int items;
    int grid;         // blocks launched (the mixed kernel strides over the items)
    int tile_group;   // mixed: observer tiles per group of the item order
    int flush_elems;  // mixed: elements summed in FP32 before the FP64 flush
    int opw;          // observers per warp
    bool tm;          // mixed: record stages copied into tensor memory and read from there
    int ring;         // mixed: bin slots per observer of the sliding ring (a power of 2), 0 = whole rows
    int ring_lo;      // mixed: slots of the smaller ring launched before this kernel in the same
                      // plan, which takes the records first when they fit it (0: none)
    size_t smem;
};

// preprocessing (tonal.cu)
struct PrepArgs {
    const float* raw;      // [surf][T][E_i][8] device
    int nsurf;
    const long long* raw_off;  // device: start (floats) of each surface's rows
    const int* e_surf;     // device: surface of each global element
    const int* e_local;    // device: element index within its surface
    const int* e_count;    // device: E_i per surface
    int E, Epad, T, nW;
    double a0, rho, pscale, cfd, dTau;
    double vinf[3];
    int periodic, lowpass;
    double gauss[13];
    double* rec64;         // [Epad][nW][5][32][4] or null
    float* rec32;          // pair-interleaved FP32 records (rec32_offset) or null
    unsigned* rmax;        // with rec32: the largest |x| (note_radius), or null
    double* fields;        // optional [E][T][18]
};
cudaError_t launch_prep(const PrepArgs& a, cudaStream_t s);

// The 16 FP32 record fields (g0..g3 above) of one element-step from the quantities of the
// preprocessing, R = double or float (the products are formed in R, then rounded).
template <typename R>
__host__ __device__ __forceinline__ void rec32_fields(const R* x, R dsD, R ATD, const R* M, const R* Md, const R* L,
                                                      const R* Ld, float* f)
{
    f[0] = (float)x[0]; f[1] = (float)x[1]; f[2] = (float)x[2]; f[3] = (float)ATD;
    f[4] = (float)M[0]; f[5] = (float)M[1]; f[6] = (float)M[2]; f[7] = (float)(dsD * Ld[0]);
    f[8] = (float)Md[0]; f[9] = (float)Md[1]; f[10] = (float)Md[2]; f[11] = (float)(dsD * Ld[1]);
    f[12] = (float)(dsD * L[0]); f[13] = (float)(dsD * L[1]); f[14] = (float)(dsD * L[2]); f[15] = (float)(dsD * Ld[2]);
}

// records straight from reference-layout AoS arrays (for the drop-in entry points)
struct AosArgs {
    const void* X;  // float or double, AoS as variables.cu:54
    const void* N;
    const void* V;
    const void* PR;
    int is_double;
    const long long* xoff;  // device per-element start of its X rows (floats)
    const long long* noff;
    const long long* voff;
    const long long* proff;
    int E, Epad, T, nW;
    double a0, rho;
    double vinf[3];
    double* rec64;
    float* rec32;
    unsigned* rmax;  // with rec32: the largest |x| (note_radius), or null
};
cudaError_t launch_aos_records(const AosArgs& a, cudaStream_t s);

// permeable preprocessing (preprocess_per) in place on reference-layout AoS arrays
constexpr int kMaxPerSteps = 4096;
struct PerArgs {
    const long long* xoff;  // device: per-element start (elements of the storage type) in Xham
    const long long* noff;  // ... in Nham
    const long long* voff;  // ... in Vham
    const long long* uoff;  // ... in Uham
    const long long* proff; // ... in PRham (4 per step)
    int E, T;
    double two_dt, inv_two_dt;                 // 2 dTau and RN(1 / (2 dTau))
    double a0, a02, rhoRef, mref2, cfd;        // a02 = pow(a0, 2), mref2 = pow(Mref, 2)
    int periodic, lowpass;
    double gauss[13];
};
cudaError_t launch_per_prep(void* X, void* N, void* V, void* U, void* PR, bool is_double, const PerArgs& a,
                            cudaStream_t s);
// the 12-column rows of a permeable deck ([surface][step][element][12], raw_off per
// surface) into FP64 AoS arrays d = X [E][T][4], N [E][T][6], V [E][T][6], U [E][T][6],
// PR [E][T][4] (derivative columns and V zero)
cudaError_t launch_per_rows(const float* raw, const long long* raw_off, const int* e_surf, const int* e_local,
                            const int* e_count, int E, int T, double* const d[5], cudaStream_t s);

struct TonalRun {
    TonalGeom g;
    TonalTile t;          // the plan; mixed with t.ring > 0: the ring kernel, then
    TonalTile wide[2];    // the wide-ring kernels (ring > 0: planned; kRingSlotsWide) for records
                          // that reach past the rings before them, and
    TonalTile rows;       // the whole-row kernel, which runs when every ring is too short
    const unsigned* rmax; // mixed: the records' largest |x| (note_radius bits)
    const void* rec;      // rec64 or rec32
    const double* obs64;  // [O][3]
    const float* obs32;
    double* acc;          // [O][T][2] (zeroed when nchunk > 1)
    DeviceErr* err;
    int precision;
};
cudaError_t plan_tonal(TonalRun& r, int W_req, int SE_req, int items_per_sm, int num_sms, size_t smem_optin,
                       int opw_req = 0, int tm_req = 0, int rows_only = 0);
cudaError_t launch_tonal(const TonalRun& r, cudaStream_t s);

// Constants of one tonal launch (one case), as the kernels read them.
struct KParams {
    const void* rec;
    int Epad, T, nW, O;
    int nW32;               // windows of the FP32 records
    int ring;               // mixed: ring slots per observer (ring kernel), 0 = whole rows
    int ring_lo;            // mixed: slots of the smaller ring launched before (TonalTile::ring_lo)
    int dual;               // mixed: ring kernels and a whole-row kernel are all launched, and
                            // each tests the records' reach
    const unsigned* rmax;   // mixed: the records' largest |x| (note_radius bits)
    double obs_rmin;        // mixed: the smallest observer distance from the origin (ring_ok)
    const float* obs32;
    const double* obs64;
    // mixed constants, as pairs (both halves equal: the operands of the packed FP32
    // instructions): -alpha, -vInf, a0, oM / dPsi.  16-byte aligned: the kernel reads
    // them two pairs at a time (measured 1.1 % slower at an 8-byte offset)
    alignas(16) float2 nalpha2;
    float2 nvx2, nvy2, nvz2, a02, kb2, alpha2;
    unsigned tmod;  // ceil(2^32 / T): bin index modulo T by multiply-high
    int toff;       // a multiple of T >= 2^23, added to bin indices before the modulo
    // FP64 constants
    double a0, alpha, ialpha, vx, vy, vz, dTau, oM, dPsi, lpi;
    int W, NS, chunk, nchunk, obs_tiles, flush_groups, tile_group;
    double* acc;
    DeviceErr* err;
};
void fill_kparams(const TonalRun& r, KParams& kp);  // of the plan r.t
void fill_kparams(const TonalRun& r, const TonalTile& tile, KParams& kp);

// Batched (persistent) mixed launch over many cases.  Work item = (case, observer tile,
// element range [e0, e1)); the kernel takes items in array order from *counter.
struct BatchItem {
    int c, ot, e0, e1;
};
// ring stages of the batched kernel: 4, or 2 for stages of 8 elements
constexpr int batch_stages(int SE) { return SE == 8 ? 2 : 4; }
// dynamic shared memory of the persistent kernel for W observers per block, elements per
// stage SE and rows of `rowlen` slots (the longest case's nTime for whole rows, the ring's
// slots for ring cases, whichever is larger)
size_t batch_smem(int W, int SE, int rowlen);
int batch_blocks_per_sm(int W, int SE, int opw, int rowlen);
size_t batch_static_smem(int SE, int opw);  // static shared memory to keep beside batch_smem
cudaError_t launch_tonal_batch(const KParams* d_cases, const BatchItem* d_items, int nitems, int* d_counter, int W,
                               int SE, int opw, int rowlen, int grid, cudaStream_t s);
constexpr int kRingSlots = 512;  // bin slots per observer of the mixed ring kernels (single deck and batched)
// Bin slots per observer of the wide rings, each for records that reach past the ring
// before it, in decks of more steps than its slots (whole rows of a shorter period hold no
// more bins).
constexpr int kWideTiers = 2;
constexpr int kRingSlotsWide[kWideTiers] = {1024, 2048};
static_assert(sizeof(TonalRun::wide) / sizeof(TonalTile) == kWideTiers, "one plan per wide ring");
// the ring that serves records of largest |x| r (ring_ok), for a deck of T steps: the
// first ring, else the first wide ring that does, else 0 (whole rows)
inline int ring_for(float r, double vx, double vy, double vz, double a0, double kb, double obs_rmin, int T)
{
    if (ring_ok(r, vx, vy, vz, a0, kb, obs_rmin, kRingSlots)) return kRingSlots;
    for (int k = 0; k < kWideTiers; ++k)
        if (T > kRingSlotsWide[k] && ring_ok(r, vx, vy, vz, a0, kb, obs_rmin, kRingSlotsWide[k]))
            return kRingSlotsWide[k];
    return 0;
}
// acc [O][T][2] of every case -> pA [T][O] (overwrite)
struct FinCase {
    const double* acc;
    double* pA;
    int O, T, tiles_o, tile0;
};
cudaError_t launch_finalize_batch(const FinCase* d_cases, int ncase, int total_tiles, cudaStream_t s);
// acc [O][T][2] -> pT/pL/pA [T][O]; mode 0 overwrite double, 1 accumulate double,
// 2 accumulate float (drop-in)
cudaError_t launch_finalize(const double* acc, int O, int T, void* pT, void* pL, void* pA, int mode,
                            cudaStream_t s);

// misc
void gauss_taps(double* w);

}  // namespace acum
