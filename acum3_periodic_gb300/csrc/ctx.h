// ctx.h -- the context behind the opaque acum_ctx handle.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <string>
#include <vector>

#include "acum_internal.h"
#include "deck.h"

namespace acum {

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t want)
    {
        if (want <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(want, 1) * sizeof(T));
        if (e == cudaSuccess) n = want;
        else p = nullptr;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// NVTX range over one ABI call (visible in Nsight timelines; a no-op otherwise)
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

struct Derived {
    double oM, dTau, dPsi, vinf[3];
};

enum {
    EV_PREP0, EV_PREP1, EV_TONAL0, EV_TONAL1, EV_FIN1, EV_BPM0, EV_BPM1, EV_ADJ0, EV_ADJ1, EV_CALL0, EV_CALL1,
    EV_BOBS0, EV_BOBS1, kNumEvents
};

int fail(struct ::acum_ctx* ctx, int code, const std::string& msg);
int cuda_fail(struct ::acum_ctx* ctx, cudaError_t e, const char* what);
void derive(const acum_inputs& in, Derived& d);
void release_bpm_state(struct ::acum_ctx* ctx);
void release_adj_state(struct ::acum_ctx* ctx);

}  // namespace acum

struct acum_ctx {
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    bool owns_stream = true;  // false for the cases of a batch, which run on its stream
    cudaEvent_t ev[acum::kNumEvents];
    std::string err;

    // deck
    bool have_deck = false;
    acum_inputs in;
    acum::Derived der;
    int nobs = 0, nsurf = 0, T = 0, nW = 0, Epad = 0;
    long long E = 0;
    std::vector<int> nelem;
    std::vector<long long> raw_off;
    size_t raw_floats = 0;
    int ncol = 8;  // floats per surface row: 8 impermeable, 12 permeable (io.cu:286, 321)
    std::vector<float> obs_file_h;
    bool have_bb = false, bb_dirty = true;
    acum::BBDeck bb;

    // device buffers
    acum::DBuf<float> d_raw;
    // pipelined runs from host rows (acum_tonal_from_host_async): two row buffers of
    // their own, a copy stream and per-buffer events; raw_cur is the buffer the
    // preprocessing reads (null: d_raw)
    acum::DBuf<float> d_raw_alt;
    float* raw_cur = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
    int async_next = 0;
    acum::DBuf<double> d_obs64;
    acum::DBuf<float> d_obs32;
    acum::DBuf<int> d_esurf, d_elocal, d_ecount;
    acum::DBuf<long long> d_rawoff, d_off;
    acum::DBuf<double> d_rec64, d_fields, d_acc, d_out;
    acum::DBuf<float> d_rec32;
    acum::DBuf<acum::DeviceErr> d_err;
    acum::DBuf<unsigned> d_rmax;  // the FP32 records' largest |x| (note_radius bits)
    double obs_rmin = -1.0;       // the observers' smallest distance from the origin (FP32 positions)
    // permeable decks: the preprocessed AoS arrays of variables.cu:54 in FP64 (X, N, V, U,
    // PR with nPRham = 4), the reference's layout (element after element, [T][width])
    acum::DBuf<double> d_per[5];
    bool per_ok = false;
    bool rec64_ok = false, rec32_ok = false;
    // layout (E, Epad, nW, T) the record buffers were last written for: the preprocessing
    // writes the real elements and steps only, so a buffer whose padding may hold records
    // of another layout is cleared first
    long long rec64_layout[4] = {-1, -1, -1, -1}, rec32_layout[4] = {-1, -1, -1, -1};

    // results kept for acum_write_outputs
    std::vector<double> h_out, h_spl, h_oaspl;
    bool have_tonal = false, have_bpm = false;

    // bookkeeping
    unsigned err_bits = 0;
    long long launches = 0;
    bool prep_timed = false, tonal_timed = false, bpm_timed = false, adj_timed = false, call_timed = false;
    int tile_W = 0, tile_SE = 0, tile_ips = 0, tile_opw = 0, tile_tm = 0, tile_rows = 0;
    acum::TonalTile last_tile, last_wide[acum::kWideTiers], last_rows;
    bool have_tonal_plan = false;

    // broadband / adjoint state lives in their own translation units
    void* bpm_state = nullptr;
    void* adj_state = nullptr;

    bool permeable() const { return in.impermeable == 0; }
    void invalidate()
    {
        rec64_ok = false;
        rec32_ok = false;
        per_ok = false;
    }
    void begin_run()
    {
        launches = 0;
        prep_timed = tonal_timed = bpm_timed = adj_timed = call_timed = false;
    }
    void release_all();
    int upload_deck_common(const acum_inputs& inp, int nob, const float* obs_file, int ns, const int* ne);
    int ensure_prep(bool need64, bool need32, bool need_fields);
    int ensure_per_prep();
    int run_tonal(int precision, double* d_pT, double* d_pL, double* d_pA);
    int finish_run();
};
