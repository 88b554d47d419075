// abi.cpp -- the C ABI of include/acum.h: contexts, deck upload, the GPU
// preprocessing and tonal runs, output writers and the reference-shaped drop-ins.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "acum_internal.h"
#include "ctx.h"
#include "deck.h"

namespace acum {

// the 1/3-octave preferred frequencies, 1 Hz .. 10 kHz, then 20 kHz (io.cu:693-699)
const double kBandHz[kBands] = {1.0,    1.25,   1.6,    2.0,    2.5,    3.15,   4.0,    5.0,    6.3,
                                8.0,    10.0,   12.5,   16.0,   20.0,   25.0,   31.5,   40.0,   50.0,
                                63.0,   80.0,   100.0,  125.0,  160.0,  200.0,  250.0,  315.0,  400.0,
                                500.0,  630.0,  800.0,  1000.0, 1250.0, 1600.0, 2000.0, 2500.0, 3150.0,
                                4000.0, 5000.0, 6300.0, 8000.0, 10000.0, 20000.0};

static thread_local std::string g_err;

int fail(acum_ctx* ctx, int code, const std::string& msg)
{
    if (ctx) ctx->err = msg;
    g_err = msg;
    return code;
}

int cuda_fail(acum_ctx* ctx, cudaError_t e, const char* what)
{
    return fail(ctx, e == cudaErrorMemoryAllocation ? ACUM_ERR_NOMEM : ACUM_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

void derive(const acum_inputs& in, Derived& d)
{
    // io.cu:73-83, evaluated in double (the FP64 build's arithmetic) from the float inputs
    d.oM = fabs(in.oM);
    d.dTau = 2 * M_PI * in.dPsi / d.oM / 360;
    d.dPsi = in.dPsi * M_PI / 180.0;
    const double xy = in.xy_angle * M_PI / 180.0, xz = in.xz_angle * M_PI / 180.0;
    d.vinf[0] = in.Minf * in.a0 * cos(xy) * cos(xz);
    d.vinf[1] = in.Minf * in.a0 * sin(xy);
    d.vinf[2] = in.Minf * in.a0 * cos(xy) * sin(xz);
}

}  // namespace acum

using namespace acum;

#define CK(ctx, call)                                         \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

// ---------------------------------------------------------------- lifecycle

void acum_ctx::release_all()
{
    d_raw.release();
    d_raw_alt.release();
    raw_cur = nullptr;
    d_obs64.release();
    d_obs32.release();
    d_esurf.release();
    d_elocal.release();
    d_ecount.release();
    d_rawoff.release();
    d_off.release();
    d_rec64.release();
    d_fields.release();
    d_acc.release();
    d_out.release();
    d_rec32.release();
    d_err.release();
    for (auto& b : d_per) b.release();
    acum::release_bpm_state(this);
    acum::release_adj_state(this);
}

extern "C" int acum_version(void) { return 1; }

extern "C" const char* acum_last_global_error(void) { return g_err.c_str(); }

extern "C" const char* acum_last_error(const acum_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

extern "C" int acum_create(acum_ctx** out, int device)
{
    if (!out) return fail(nullptr, ACUM_ERR_INVALID, "acum_create: null out");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(nullptr, ACUM_ERR_CUDA, "acum_create: no CUDA device");
    if (device < 0 || device >= ndev) return fail(nullptr, ACUM_ERR_INVALID, "acum_create: bad device index");
    std::unique_ptr<acum_ctx> c(new acum_ctx());
    c->device = device;
    DeviceGuard g(device);
    CK(nullptr, cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    int optin = 0;
    CK(nullptr, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    c->smem_optin = (size_t)optin;
    CK(nullptr, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    for (int i = 0; i < kNumEvents; ++i) CK(nullptr, cudaEventCreate(&c->ev[i]));
    CK(nullptr, c->d_err.ensure(1));
    CK(nullptr, cudaMemset(c->d_err.p, 0, sizeof(DeviceErr)));
    *out = c.release();
    return ACUM_OK;
}

extern "C" int acum_destroy(acum_ctx* ctx)
{
    if (!ctx) return ACUM_OK;
    {
        DeviceGuard g(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        ctx->release_all();
        for (int i = 0; i < kNumEvents; ++i) cudaEventDestroy(ctx->ev[i]);
        if (ctx->owns_stream) cudaStreamDestroy(ctx->stream);
        if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
        for (int k = 0; k < 2; ++k) {
            if (ctx->ev_copied[k]) cudaEventDestroy(ctx->ev_copied[k]);
            if (ctx->ev_free[k]) cudaEventDestroy(ctx->ev_free[k]);
        }
    }
    delete ctx;
    return ACUM_OK;
}

// --------------------------------------------------------------------- deck

int acum_ctx::upload_deck_common(const acum_inputs& inp, int nob, const float* obs_file, int ns, const int* ne)
{
    if (inp.nTime < 6) return fail(this, ACUM_ERR_INVALID, "nTime must be at least 6");
    if (nob <= 0) return fail(this, ACUM_ERR_INVALID, "no observers");
    if (ns <= 0) return fail(this, ACUM_ERR_INVALID, "no surfaces");
    if (inp.impermeable == 0 && inp.nTime > kMaxPerSteps)
        return fail(this, ACUM_ERR_UNSUPPORTED, "permeable decks: at most 4096 steps per period");
    if (inp.oM == 0.0 || inp.dPsi == 0.0) return fail(this, ACUM_ERR_INVALID, "oM and dPsi must be non-zero");
    in = inp;
    derive(in, der);
    ncol = surface_columns(in.impermeable);
    nobs = nob;
    nsurf = ns;
    nelem.assign(ne, ne + ns);
    E = 0;
    raw_off.assign(ns, 0);
    long long off = 0;
    for (int i = 0; i < ns; ++i) {
        if (nelem[i] < 0) return fail(this, ACUM_ERR_INVALID, "negative element count");
        raw_off[i] = off;
        off += (long long)in.nTime * nelem[i] * ncol;
        E += nelem[i];
    }
    if (E <= 0) return fail(this, ACUM_ERR_INVALID, "no elements");
    raw_floats = (size_t)off;
    T = in.nTime;
    nW = (T + kWin - 1) / kWin;
    Epad = (int)((E + 7) / 8 * 8);  // a multiple of every elements-per-stage
    // observers: rObs = obs.dat * OBSscale (io.cu:123-128)
    obs_file_h.assign(obs_file, obs_file + 3 * (size_t)nob);
    std::vector<double> o64(3 * (size_t)nob);
    std::vector<float> o32(3 * (size_t)nob);
    for (size_t i = 0; i < o64.size(); ++i) {
        o64[i] = (double)obs_file[i] * in.OBSscale;
        o32[i] = (float)o64[i];
    }
    obs_rmin = obs_min_distance(o32.data(), nob);
    DeviceGuard g(device);
    CK(this, d_obs64.ensure(o64.size()));
    CK(this, d_obs32.ensure(o32.size()));
    CK(this, cudaMemcpy(d_obs64.p, o64.data(), o64.size() * 8, cudaMemcpyHostToDevice));
    CK(this, cudaMemcpy(d_obs32.p, o32.data(), o32.size() * 4, cudaMemcpyHostToDevice));
    // element -> (surface, local index)
    std::vector<int> es((size_t)E), el((size_t)E);
    long long k = 0;
    for (int i = 0; i < ns; ++i)
        for (int j = 0; j < nelem[i]; ++j, ++k) {
            es[k] = i;
            el[k] = j;
        }
    CK(this, d_esurf.ensure(E));
    CK(this, d_elocal.ensure(E));
    CK(this, d_ecount.ensure(ns));
    CK(this, d_rawoff.ensure(ns));
    CK(this, cudaMemcpy(d_esurf.p, es.data(), E * 4, cudaMemcpyHostToDevice));
    CK(this, cudaMemcpy(d_elocal.p, el.data(), E * 4, cudaMemcpyHostToDevice));
    CK(this, cudaMemcpy(d_ecount.p, nelem.data(), ns * 4, cudaMemcpyHostToDevice));
    CK(this, cudaMemcpy(d_rawoff.p, raw_off.data(), ns * 8, cudaMemcpyHostToDevice));
    CK(this, d_raw.ensure(raw_floats));
    have_deck = true;
    invalidate();
    per_ok = false;
    have_bb = false;
    have_tonal = false;
    have_bpm = false;
    return ACUM_OK;
}

extern "C" int acum_set_deck(acum_ctx* ctx, const acum_inputs* in, int nobs, const float* obs_file, int nsurf,
                             const int* nelem, const float* raw, int raw_on_device)
{
    acum::NvtxRange nvtx_range_("acum_set_deck");
    if (!ctx || !in || !obs_file || !nelem || !raw) return fail(ctx, ACUM_ERR_INVALID, "acum_set_deck: null argument");
    int rc = ctx->upload_deck_common(*in, nobs, obs_file, nsurf, nelem);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    CK(ctx, cudaMemcpyAsync(ctx->d_raw.p, raw, ctx->raw_floats * 4,
                            raw_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return ACUM_OK;
}

extern "C" int acum_update_surfaces(acum_ctx* ctx, const float* raw, int raw_on_device)
{
    if (!ctx || !raw) return fail(ctx, ACUM_ERR_INVALID, "acum_update_surfaces: null argument");
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    DeviceGuard g(ctx->device);
    CK(ctx, cudaMemcpyAsync(ctx->d_raw.p, raw, ctx->raw_floats * 4,
                            raw_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
    ctx->invalidate();
    return ACUM_OK;
}

extern "C" int acum_read_deck_sizes(const char* dir, long long* out)
{
    acum::NvtxRange nvtx_range_("acum_read_deck_sizes");
    if (!dir || !out) return fail(nullptr, ACUM_ERR_INVALID, "acum_read_deck_sizes: null argument");
    std::string d(dir), err;
    acum_inputs in;
    int ns = 0, nob = 0;
    std::vector<float> obs, raw;
    std::vector<int> ne;
    if (!read_inputs(d, in, ns, &err)) return fail(nullptr, ACUM_ERR_IO, err);
    BBDeck bb;
    if (in.BB_noise == 1 && !read_bb(d, ns, in.nTime, bb, &err)) return fail(nullptr, ACUM_ERR_IO, err);
    if (!read_observers(d, obs, nob, &err)) return fail(nullptr, ACUM_ERR_IO, err);
    if (!read_surfaces(d, ns, in.nTime, surface_columns(in.impermeable), ne, raw, &err))
        return fail(nullptr, ACUM_ERR_IO, err);
    long long E = 0, bbs = 0;
    for (int x : ne) E += x;
    for (int n : bb.nsect) bbs += n;
    out[0] = ns;
    out[1] = in.nTime;
    out[2] = nob;
    out[3] = E;
    out[4] = in.BB_noise == 1 ? bbs : 0;
    out[5] = in.BB_noise == 1 ? 1 : 0;
    return ACUM_OK;
}

extern "C" int acum_write_surface_cache(const char* dir)
{
    acum::NvtxRange nvtx_range_("acum_write_surface_cache");
    if (!dir) return fail(nullptr, ACUM_ERR_INVALID, "acum_write_surface_cache: null argument");
    std::string d(dir), err;
    acum_inputs in;
    int ns = 0;
    std::vector<float> raw;
    std::vector<int> ne;
    if (!read_inputs(d, in, ns, &err)) return fail(nullptr, ACUM_ERR_IO, err);
    const int ncol = surface_columns(in.impermeable);
    if (!read_surfaces(d, ns, in.nTime, ncol, ne, raw, &err)) return fail(nullptr, ACUM_ERR_IO, err);
    if (!write_surface_cache(d, ns, in.nTime, ncol, ne, raw, &err)) return fail(nullptr, ACUM_ERR_IO, err);
    return ACUM_OK;
}

extern "C" int acum_load_deck(acum_ctx* ctx, const char* dir)
{
    acum::NvtxRange nvtx_range_("acum_load_deck");
    if (!ctx || !dir) return fail(ctx, ACUM_ERR_INVALID, "acum_load_deck: null argument");
    std::string d(dir), err;
    acum_inputs in;
    int ns = 0, nob = 0;
    std::vector<float> obs, raw;
    std::vector<int> ne;
    if (!read_inputs(d, in, ns, &err)) return fail(ctx, ACUM_ERR_IO, err);
    BBDeck bb;
    if (in.BB_noise == 1 && !read_bb(d, ns, in.nTime, bb, &err)) return fail(ctx, ACUM_ERR_IO, err);
    if (!read_observers(d, obs, nob, &err)) return fail(ctx, ACUM_ERR_IO, err);
    if (!read_surfaces(d, ns, in.nTime, surface_columns(in.impermeable), ne, raw, &err))
        return fail(ctx, ACUM_ERR_IO, err);
    int rc = acum_set_deck(ctx, &in, nob, obs.data(), ns, ne.data(), raw.data(), 0);
    if (rc) return rc;
    if (in.BB_noise == 1) {
        ctx->bb = std::move(bb);
        ctx->have_bb = true;
        ctx->bb_dirty = true;
    }
    return ACUM_OK;
}

extern "C" int acum_get_sizes(const acum_ctx* ctx, long long* out)
{
    if (!ctx || !out) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return ACUM_ERR_STATE;
    long long bbs = 0;
    for (int n : ctx->bb.nsect) bbs += n;
    out[0] = ctx->nsurf;
    out[1] = ctx->T;
    out[2] = ctx->nobs;
    out[3] = ctx->E;
    out[4] = ctx->have_bb ? bbs : 0;
    out[5] = ctx->have_bb ? 1 : 0;
    return ACUM_OK;
}

extern "C" int acum_last_plan(const acum_ctx* ctx, int* out)
{
    if (!ctx || !out) return ACUM_ERR_INVALID;
    if (!ctx->have_tonal_plan) return ACUM_ERR_STATE;
    const TonalTile& t = ctx->last_tile;
    out[0] = t.W;
    out[1] = t.SE;
    out[2] = t.NS;
    out[3] = t.chunk;
    out[4] = t.nchunk;
    out[5] = t.items;
    out[6] = t.opw;
    out[7] = t.tm ? 1 : 0;
    return ACUM_OK;
}

extern "C" int acum_set_tile(acum_ctx* ctx, int obs_per_block, int elems_per_stage, int items_per_sm)
{
    if (!ctx) return ACUM_ERR_INVALID;
    if (obs_per_block < 0 || obs_per_block > 32 || items_per_sm < 0 || items_per_sm > 64 ||
        (elems_per_stage != 0 && elems_per_stage != 2 && elems_per_stage != 4 && elems_per_stage != 8))
        return fail(ctx, ACUM_ERR_INVALID, "acum_set_tile: out of range");
    ctx->tile_W = obs_per_block;
    ctx->tile_SE = elems_per_stage;
    ctx->tile_ips = items_per_sm;
    return ACUM_OK;
}

extern "C" int acum_set_tensor_memory(acum_ctx* ctx, int use)
{
    if (!ctx) return ACUM_ERR_INVALID;
    if (use < 0 || use > 2) return fail(ctx, ACUM_ERR_INVALID, "acum_set_tensor_memory: out of range");
    ctx->tile_tm = use;
    return ACUM_OK;
}

extern "C" int acum_set_obs_per_warp(acum_ctx* ctx, int obs_per_warp)
{
    if (!ctx) return ACUM_ERR_INVALID;
    if (obs_per_warp < 0 || obs_per_warp > 2) return fail(ctx, ACUM_ERR_INVALID, "acum_set_obs_per_warp: out of range");
    ctx->tile_opw = obs_per_warp;
    return ACUM_OK;
}

extern "C" int acum_set_ring(acum_ctx* ctx, int mode)
{
    if (!ctx) return ACUM_ERR_INVALID;
    if (mode < 0 || mode > 1) return fail(ctx, ACUM_ERR_INVALID, "acum_set_ring: out of range");
    ctx->tile_rows = mode;
    return ACUM_OK;
}

extern "C" int acum_last_plan_ring(acum_ctx* ctx, int* out)
{
    if (!ctx || !out) return ACUM_ERR_INVALID;
    if (!ctx->have_tonal_plan) return ACUM_ERR_STATE;
    out[0] = ctx->last_tile.ring;
    out[1] = ctx->last_rows.W;
    out[2] = ctx->last_rows.SE;
    out[3] = ctx->last_rows.NS;
    out[4] = 0;
    for (int k = 0; k < kWideTiers; ++k) {
        out[5 + 3 * k] = ctx->last_wide[k].ring;
        out[6 + 3 * k] = ctx->last_wide[k].W;
        out[7 + 3 * k] = ctx->last_wide[k].NS;
    }
    if (ctx->last_tile.ring > 0) {
        // the tests the kernels make, from the same radius
        DeviceGuard g(ctx->device);
        unsigned bits = 0;
        CK(ctx, cudaStreamSynchronize(ctx->stream));
        CK(ctx, cudaMemcpy(&bits, ctx->d_rmax.p, sizeof(bits), cudaMemcpyDeviceToHost));
        float r;
        memcpy(&r, &bits, sizeof(r));
        const double kb = ctx->der.oM / ctx->der.dPsi;
        int rings[1 + kWideTiers] = {ctx->last_tile.ring};
        for (int k = 0; k < kWideTiers; ++k) rings[1 + k] = ctx->last_wide[k].ring;
        for (int R : rings)
            if (R > 0 && ring_ok(r, ctx->der.vinf[0], ctx->der.vinf[1], ctx->der.vinf[2], ctx->in.a0, kb,
                                 ctx->obs_rmin, R)) {
                out[4] = R;
                break;
            }
    }
    return ACUM_OK;
}

// ------------------------------------------------------------ preprocessing

int acum_ctx::ensure_prep(bool need64, bool need32, bool need_fields)
{
    DeviceGuard g(device);
    if (permeable())
        return fail(this, ACUM_ERR_UNSUPPORTED,
                    "a permeable deck (impermeable 0) has no impermeable records or fields: the reference "
                    "runs no acoustic kernel for it (main.cu:236); acum_get_permeable_fields gives its "
                    "preprocessed arrays");
    const bool do64 = need64 && !rec64_ok, do32 = need32 && !rec32_ok;
    if (!do64 && !do32 && !need_fields) return ACUM_OK;
    if (!d_raw.p) return fail(this, ACUM_ERR_STATE, "the surface rows were released after preprocessing");
    if (T > 4096) return fail(this, ACUM_ERR_UNSUPPORTED, "nTime above 4096 is not supported by the preprocessing");
    const size_t nrec = (size_t)Epad * nW * kGroups * kWin * 4;     // FP64 records
    const size_t nrec32 = (size_t)Epad * nwin32(T) * kGroups32 * kWin * 4;  // FP32 records
    const long long layout[4] = {(long long)E, (long long)Epad, (long long)nW, (long long)T};
    const auto same = [&](const long long* l) { return std::equal(l, l + 4, layout); };
    if (do64) {
        const bool clear = d_rec64.n < nrec || !same(rec64_layout);
        CK(this, d_rec64.ensure(nrec));
        if (clear) CK(this, cudaMemsetAsync(d_rec64.p, 0, nrec * 8, stream));
        std::copy(layout, layout + 4, rec64_layout);
    }
    if (do32) {
        const bool clear = d_rec32.n < nrec32 || !same(rec32_layout);
        CK(this, d_rec32.ensure(nrec32));
        if (clear) CK(this, cudaMemsetAsync(d_rec32.p, 0, nrec32 * 4, stream));
        std::copy(layout, layout + 4, rec32_layout);
        CK(this, d_rmax.ensure(1));
        CK(this, cudaMemsetAsync(d_rmax.p, 0, sizeof(unsigned), stream));
    }
    if (need_fields) CK(this, d_fields.ensure((size_t)E * T * kFields));
    PrepArgs a;
    memset(&a, 0, sizeof(a));
    a.raw = raw_cur ? raw_cur : d_raw.p;
    a.nsurf = nsurf;
    a.raw_off = d_rawoff.p;
    a.e_surf = d_esurf.p;
    a.e_local = d_elocal.p;
    a.e_count = d_ecount.p;
    a.E = (int)E;
    a.Epad = Epad;
    a.T = T;
    a.nW = nW;
    a.a0 = in.a0;
    a.rho = in.rhoRef;
    for (int c = 0; c < 3; ++c) a.vinf[c] = der.vinf[c];
    a.pscale = 0.5 * in.rhoRef * (in.Mref * in.Mref) * (in.a0 * in.a0);
    a.cfd = in.CFDscale;
    a.dTau = der.dTau;
    a.periodic = in.periodic;
    a.lowpass = in.lowpass;
    gauss_taps(a.gauss);
    // the FP32 records always come from the FP32 preprocessing (the same records whatever
    // else was asked for before); the FP64 records and the fields from the FP64 one
    CK(this, cudaEventRecord(ev[EV_PREP0], stream));
    if (do32) {
        PrepArgs a32 = a;
        a32.rec64 = nullptr;
        a32.fields = nullptr;
        a32.rec32 = d_rec32.p;
        a32.rmax = d_rmax.p;
        CK(this, launch_prep(a32, stream));
        launches += 1;
    }
    if (do64 || need_fields) {
        a.rec64 = do64 ? d_rec64.p : nullptr;
        a.rec32 = nullptr;
        a.fields = need_fields ? d_fields.p : nullptr;
        CK(this, launch_prep(a, stream));
        launches += 1;
    }
    CK(this, cudaEventRecord(ev[EV_PREP1], stream));
    prep_timed = true;
    if (do64) rec64_ok = true;
    if (do32) rec32_ok = true;
    return ACUM_OK;
}

extern "C" int acum_preprocess(acum_ctx* ctx)
{
    acum::NvtxRange nvtx_range_("acum_preprocess");
    if (!ctx) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    ctx->begin_run();
    int rc = ctx->permeable() ? ctx->ensure_per_prep() : ctx->ensure_prep(true, true, false);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return ACUM_OK;
}

extern "C" int acum_get_fields(acum_ctx* ctx, double* host_fields)
{
    if (!ctx || !host_fields) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    ctx->begin_run();
    int rc = ctx->ensure_prep(false, false, true);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    CK(ctx, cudaMemcpyAsync(host_fields, ctx->d_fields.p, (size_t)ctx->E * ctx->T * kFields * 8,
                            cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return ACUM_OK;
}

// --------------------------------------------------------------------- tonal

int acum_ctx::run_tonal(int precision, double* d_pT, double* d_pL, double* d_pA)
{
    if (precision != ACUM_PLAIN_FP64 && precision != ACUM_MIXED)
        return fail(this, ACUM_ERR_INVALID, "precision must be ACUM_PLAIN_FP64 or ACUM_MIXED");
    const bool f64 = precision == ACUM_PLAIN_FP64;
    if (permeable()) {
        // main.cu:87 preprocesses a permeable deck and main.cu:236 launches the kernel only
        // for impermeable ones: the pressures stay as main.cu:123-130 zeroed them
        int rc = ensure_per_prep();
        if (rc) return rc;
        DeviceGuard g(device);
        const size_t n = (size_t)T * nobs * sizeof(double);
        for (double* o : {d_pT, d_pL, d_pA})
            if (o) CK(this, cudaMemsetAsync(o, 0, n, stream));
        return ACUM_OK;
    }
    int rc = ensure_prep(f64, !f64, false);
    if (rc) return rc;
    DeviceGuard g(device);
    TonalRun r;
    memset(&r, 0, sizeof(r));
    r.g.E = (int)E;
    r.g.Epad = Epad;
    r.g.T = T;
    r.g.nW = nW;
    r.g.O = nobs;
    r.g.a0 = in.a0;
    r.g.rho = in.rhoRef;
    r.g.oM = der.oM;
    r.g.dPsi = der.dPsi;
    r.g.dTau = der.dTau;
    r.g.lpi = T * der.dPsi;
    for (int c = 0; c < 3; ++c) r.g.vinf[c] = der.vinf[c];
    r.g.obs_rmin = obs_rmin;
    r.precision = precision;
    r.rmax = f64 ? nullptr : d_rmax.p;
    CK(this, plan_tonal(r, tile_W, tile_SE, tile_ips, num_sms, smem_optin, tile_opw, tile_tm, tile_rows));
    r.rec = f64 ? (const void*)d_rec64.p : (const void*)d_rec32.p;
    r.obs64 = d_obs64.p;
    r.obs32 = d_obs32.p;
    CK(this, d_acc.ensure((size_t)nobs * T * 2));
    r.acc = d_acc.p;
    r.err = d_err.p;
    last_tile = r.t;
    for (int k = 0; k < kWideTiers; ++k) last_wide[k] = r.wide[k];
    last_rows = r.rows;
    have_tonal_plan = true;
    // the mixed form always adds into the FP64 sums; the FP64 form stores when one block
    // owns an observer's whole element range
    if (r.t.nchunk > 1 || !f64) CK(this, cudaMemsetAsync(d_acc.p, 0, (size_t)nobs * T * 2 * 8, stream));
    CK(this, cudaEventRecord(ev[EV_TONAL0], stream));
    CK(this, launch_tonal(r, stream));
    CK(this, cudaEventRecord(ev[EV_TONAL1], stream));
    CK(this, launch_finalize(d_acc.p, nobs, T, d_pT, d_pL, d_pA, 0, stream));
    CK(this, cudaEventRecord(ev[EV_FIN1], stream));
    launches += r.t.ring > 0 ? 3 : 2;
    for (int k = 0; k < kWideTiers; ++k) launches += r.wide[k].ring > 0 ? 1 : 0;
    tonal_timed = true;
    return ACUM_OK;
}

int acum_ctx::finish_run()
{
    DeviceGuard g(device);
    CK(this, cudaStreamSynchronize(stream));
    DeviceErr h;
    CK(this, cudaMemcpy(&h, d_err.p, sizeof(h), cudaMemcpyDeviceToHost));
    err_bits |= h.bits;
    if (h.bits & ACUM_DEVERR_TIMEOUT) {
        cudaMemset(d_err.p, 0, sizeof(DeviceErr));
        return fail(this, ACUM_ERR_TIMEOUT, "a bounded shared-memory pipeline wait ran out; results are incomplete");
    }
    return ACUM_OK;
}

extern "C" int acum_tonal_device(acum_ctx* ctx, int precision, double* d_pT, double* d_pL, double* d_pA)
{
    acum::NvtxRange nvtx_range_("acum_tonal_device");
    if (!ctx) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    ctx->begin_run();
    if (!d_pT && !d_pL && !d_pA) {
        // results stay in the context's own output buffer
        const size_t n = (size_t)ctx->T * ctx->nobs;
        DeviceGuard g(ctx->device);
        CK(ctx, ctx->d_out.ensure(3 * n));
        return ctx->run_tonal(precision, ctx->d_out.p, ctx->d_out.p + n, ctx->d_out.p + 2 * n);
    }
    return ctx->run_tonal(precision, d_pT, d_pL, d_pA);
}

extern "C" int acum_surfaces_device_ptr(acum_ctx* ctx, float** p)
{
    if (!ctx || !p) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    *p = ctx->d_raw.p;
    return ACUM_OK;
}

extern "C" int acum_mark_surfaces_changed(acum_ctx* ctx)
{
    if (!ctx) return ACUM_ERR_INVALID;
    ctx->invalidate();
    return ACUM_OK;
}

extern "C" int acum_stream(acum_ctx* ctx, void** stream)
{
    if (!ctx || !stream) return ACUM_ERR_INVALID;
    *stream = (void*)ctx->stream;
    return ACUM_OK;
}

extern "C" int acum_sync(acum_ctx* ctx)
{
    if (!ctx) return ACUM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->copy_stream) CK(ctx, cudaStreamSynchronize(ctx->copy_stream));
    return ctx->finish_run();
}

extern "C" int acum_tonal_from_host_async(acum_ctx* ctx, int precision, const float* raw, double* pA_host)
{
    acum::NvtxRange nvtx_range_("acum_tonal_from_host_async");
    if (!ctx || !raw || !pA_host) return fail(ctx, ACUM_ERR_INVALID, "acum_tonal_from_host_async: null argument");
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    DeviceGuard g(ctx->device);
    if (!ctx->copy_stream) {
        CK(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            CK(ctx, cudaEventCreateWithFlags(&ctx->ev_copied[k], cudaEventDisableTiming));
            CK(ctx, cudaEventCreateWithFlags(&ctx->ev_free[k], cudaEventDisableTiming));
            CK(ctx, cudaEventRecord(ctx->ev_free[k], ctx->stream));
        }
    }
    CK(ctx, ctx->d_raw_alt.ensure(2 * ctx->raw_floats));
    const int b = ctx->async_next;
    ctx->async_next ^= 1;
    float* buf = ctx->d_raw_alt.p + (size_t)b * ctx->raw_floats;
    const size_t n = (size_t)ctx->T * ctx->nobs;
    CK(ctx, ctx->d_out.ensure(3 * n));
    // the copy of this call's rows waits only for the run that last read the same buffer,
    // so it overlaps the previous call's compute
    CK(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_free[b], 0));
    CK(ctx, cudaMemcpyAsync(buf, raw, ctx->raw_floats * 4, cudaMemcpyHostToDevice, ctx->copy_stream));
    CK(ctx, cudaEventRecord(ctx->ev_copied[b], ctx->copy_stream));
    CK(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[b], 0));
    ctx->begin_run();
    ctx->raw_cur = buf;
    ctx->invalidate();
    int rc = ctx->run_tonal(precision, nullptr, nullptr, ctx->d_out.p + 2 * n);
    ctx->raw_cur = nullptr;
    ctx->invalidate();  // the records now hold this buffer's rows, not d_raw's
    if (rc) return rc;
    CK(ctx, cudaEventRecord(ctx->ev_free[b], ctx->stream));
    CK(ctx, cudaMemcpyAsync(pA_host, ctx->d_out.p + 2 * n, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return ACUM_OK;
}

extern "C" int acum_tonal(acum_ctx* ctx, int precision, double* pT, double* pL, double* pA)
{
    acum::NvtxRange nvtx_range_("acum_tonal");
    if (!ctx) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    DeviceGuard g(ctx->device);
    const size_t n = (size_t)ctx->T * ctx->nobs;
    CK(ctx, ctx->d_out.ensure(3 * n));
    ctx->begin_run();
    CK(ctx, cudaEventRecord(ctx->ev[EV_CALL0], ctx->stream));
    int rc = ctx->run_tonal(precision, ctx->d_out.p, ctx->d_out.p + n, ctx->d_out.p + 2 * n);
    if (rc) return rc;
    ctx->h_out.resize(3 * n);
    CK(ctx, cudaMemcpyAsync(ctx->h_out.data(), ctx->d_out.p, 3 * n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaEventRecord(ctx->ev[EV_CALL1], ctx->stream));
    ctx->call_timed = true;
    rc = ctx->finish_run();
    if (rc) return rc;
    if (pT) memcpy(pT, ctx->h_out.data(), n * 8);
    if (pL) memcpy(pL, ctx->h_out.data() + n, n * 8);
    if (pA) memcpy(pA, ctx->h_out.data() + 2 * n, n * 8);
    ctx->have_tonal = true;
    return ACUM_OK;
}

extern "C" int acum_tonal_from_host(acum_ctx* ctx, int precision, const float* raw, double* pA_host)
{
    acum::NvtxRange nvtx_range_("acum_tonal_from_host");
    if (!ctx || !raw || !pA_host) return fail(ctx, ACUM_ERR_INVALID, "acum_tonal_from_host: null argument");
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    DeviceGuard g(ctx->device);
    const size_t n = (size_t)ctx->T * ctx->nobs;
    CK(ctx, ctx->d_out.ensure(3 * n));
    ctx->begin_run();
    CK(ctx, cudaEventRecord(ctx->ev[EV_CALL0], ctx->stream));
    CK(ctx, cudaMemcpyAsync(ctx->d_raw.p, raw, ctx->raw_floats * 4, cudaMemcpyHostToDevice, ctx->stream));
    ctx->invalidate();
    int rc = ctx->run_tonal(precision, nullptr, nullptr, ctx->d_out.p + 2 * n);
    if (rc) return rc;
    CK(ctx, cudaMemcpyAsync(pA_host, ctx->d_out.p + 2 * n, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaEventRecord(ctx->ev[EV_CALL1], ctx->stream));
    ctx->call_timed = true;
    return ctx->finish_run();
}

extern "C" int acum_device_error_word(acum_ctx* ctx, uint32_t* out, int reset)
{
    if (!ctx || !out) return ACUM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    DeviceErr h;
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    CK(ctx, cudaMemcpy(&h, ctx->d_err.p, sizeof(h), cudaMemcpyDeviceToHost));
    *out = h.bits | ctx->err_bits;
    if (reset) {
        CK(ctx, cudaMemset(ctx->d_err.p, 0, sizeof(DeviceErr)));
        ctx->err_bits = 0;
    }
    return ACUM_OK;
}

extern "C" int acum_last_timing(const acum_ctx* ctx, int which, double* ms, long long* launches)
{
    if (!ctx || !ms) return ACUM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    *ms = -1.0;
    if (launches) *launches = ctx->launches;
    int a = -1, b = -1;
    bool have = false;
    switch (which) {
    case 0: a = EV_TONAL0; b = EV_TONAL1; have = ctx->tonal_timed; break;
    case 1: a = EV_PREP0; b = EV_PREP1; have = ctx->prep_timed; break;
    case 2: a = EV_TONAL1; b = EV_FIN1; have = ctx->tonal_timed; break;
    case 3: a = EV_BPM0; b = EV_BPM1; have = ctx->bpm_timed; break;
    case 4: a = EV_ADJ0; b = EV_ADJ1; have = ctx->adj_timed; break;
    case 5: a = EV_CALL0; b = EV_CALL1; have = ctx->call_timed; break;
    case 6: a = EV_BOBS0; b = EV_BOBS1; have = ctx->bpm_timed; break;
    default: return ACUM_ERR_INVALID;
    }
    if (!have) return ACUM_ERR_STATE;
    if (cudaEventSynchronize(ctx->ev[b]) != cudaSuccess) return ACUM_ERR_CUDA;
    float f = 0.f;
    if (cudaEventElapsedTime(&f, ctx->ev[a], ctx->ev[b]) != cudaSuccess) return ACUM_ERR_CUDA;
    *ms = f;
    return ACUM_OK;
}

extern "C" int acum_write_outputs(acum_ctx* ctx, const char* dir)
{
    acum::NvtxRange nvtx_range_("acum_write_outputs");
    if (!ctx || !dir) return ACUM_ERR_INVALID;
    std::string err;
    if (ctx->have_tonal) {
        const size_t n = (size_t)ctx->T * ctx->nobs;
        if (!write_time_history(dir, ctx->T, ctx->nobs, ctx->in.dPsi, ctx->h_out.data(), ctx->h_out.data() + n,
                                ctx->h_out.data() + 2 * n, &err))
            return fail(ctx, ACUM_ERR_IO, err);
    }
    if (ctx->have_bpm) {
        if (!write_bb_output(dir, ctx->nobs, ctx->h_oaspl.data(), ctx->h_spl.data(), kBandHz, kBands, &err))
            return fail(ctx, ACUM_ERR_IO, err);
    }
    if (!ctx->have_tonal && !ctx->have_bpm) return fail(ctx, ACUM_ERR_STATE, "nothing computed yet");
    return ACUM_OK;
}

extern "C" int acum_host_alloc(void** p, size_t bytes)
{
    if (!p) return ACUM_ERR_INVALID;
    cudaError_t e = cudaHostAlloc(p, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaHostAlloc");
    return ACUM_OK;
}

extern "C" int acum_host_free(void* p)
{
    if (!p) return ACUM_OK;
    cudaError_t e = cudaFreeHost(p);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaFreeHost");
    return ACUM_OK;
}

// ------------------------------------------------------------------ drop-ins

namespace {

// One internal context per device serves the reference-shaped calls; it only holds
// scratch buffers (records, sums) between calls.
std::mutex g_dropin_mu;
std::map<int, acum_ctx*> g_dropin;

acum_ctx* dropin_ctx(int dev)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    auto it = g_dropin.find(dev);
    if (it != g_dropin.end()) return it->second;
    acum_ctx* c = nullptr;
    if (acum_create(&c, dev) != ACUM_OK) return nullptr;
    g_dropin[dev] = c;
    return c;
}

template <typename S>
int find_pth(const S* rObs, const S* tObs, S* pT, S* pL, S* pA, const S* Xham, const S* Nham, const S* Vham,
             const S* PRham, int nSurf, const int* XPtr, const int* NPtr, const int* VPtr, const int* PRPtr,
             const int* Ecnt, int nObs, int nTime, double dPsi, double dTau, double a0, double rhoRef, const S* vInf,
             double oM, void* stream_v)
{
    const bool f64 = sizeof(S) == 8;
    if (!rObs || !tObs || !Xham || !Nham || !Vham || !PRham || !XPtr || !NPtr || !VPtr || !PRPtr || !Ecnt || !vInf)
        return fail(nullptr, ACUM_ERR_INVALID, "findPressureTimeHistory: null argument");
    if (nSurf <= 0 || nObs <= 0 || nTime < 4) return fail(nullptr, ACUM_ERR_INVALID, "findPressureTimeHistory: sizes");
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_fail(nullptr, ce, "cudaGetDevice");
    acum_ctx* c = dropin_ctx(dev);
    if (!c) return fail(nullptr, ACUM_ERR_CUDA, "findPressureTimeHistory: cannot create a context");
    cudaStream_t st = stream_v ? (cudaStream_t)stream_v : (cudaStream_t)0;
    // the small per-surface arrays and the bin grid live in device memory, as the
    // reference passes them
    std::vector<int> hE(nSurf), hX(nSurf), hN(nSurf), hV(nSurf), hP(nSurf);
    std::vector<S> hv(3), ht(nTime);
    CK(nullptr, cudaMemcpyAsync(hE.data(), Ecnt, nSurf * 4, cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaMemcpyAsync(hX.data(), XPtr, nSurf * 4, cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaMemcpyAsync(hN.data(), NPtr, nSurf * 4, cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaMemcpyAsync(hV.data(), VPtr, nSurf * 4, cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaMemcpyAsync(hP.data(), PRPtr, nSurf * 4, cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaMemcpyAsync(hv.data(), vInf, 3 * sizeof(S), cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaMemcpyAsync(ht.data(), tObs, nTime * sizeof(S), cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaStreamSynchronize(st));
    // the walk of core.cu:199-231 assumes the uniform grid main.cu:124 builds
    for (int t = 0; t < nTime; ++t) {
        const double want = (double)(S)(t * (S)dPsi);
        if (fabs((double)ht[t] - want) > 1e-6 * fabs(dPsi) * (1 + t))
            return fail(nullptr, ACUM_ERR_UNSUPPORTED, "findPressureTimeHistory: tObs must be t*dPsi");
    }
    long long E = 0;
    for (int i = 0; i < nSurf; ++i) E += hE[i];
    if (E <= 0) return fail(nullptr, ACUM_ERR_INVALID, "findPressureTimeHistory: no elements");
    std::vector<long long> xo(E), no(E), vo(E), po(E);
    long long k = 0;
    for (int i = 0; i < nSurf; ++i)
        for (int j = 0; j < hE[i]; ++j, ++k) {
            xo[k] = hX[i] + (long long)j * nTime * 4;
            no[k] = hN[i] + (long long)j * nTime * 6;
            vo[k] = hV[i] + (long long)j * nTime * 6;
            po[k] = hP[i] + (long long)j * nTime * 2;
        }
    const int nW = (nTime + kWin - 1) / kWin;
    const int Epad = (int)((E + 7) / 8 * 8);
    CK(nullptr, c->d_off.ensure(4 * (size_t)E));
    CK(nullptr, cudaMemcpyAsync(c->d_off.p, xo.data(), E * 8, cudaMemcpyHostToDevice, st));
    CK(nullptr, cudaMemcpyAsync(c->d_off.p + E, no.data(), E * 8, cudaMemcpyHostToDevice, st));
    CK(nullptr, cudaMemcpyAsync(c->d_off.p + 2 * E, vo.data(), E * 8, cudaMemcpyHostToDevice, st));
    CK(nullptr, cudaMemcpyAsync(c->d_off.p + 3 * E, po.data(), E * 8, cudaMemcpyHostToDevice, st));
    const size_t nrec = f64 ? (size_t)Epad * nW * kGroups * kWin * 4 : (size_t)Epad * nwin32(nTime) * kGroups32 * kWin * 4;
    AosArgs a;
    memset(&a, 0, sizeof(a));
    a.X = Xham;
    a.N = Nham;
    a.V = Vham;
    a.PR = PRham;
    a.is_double = f64;
    a.xoff = c->d_off.p;
    a.noff = c->d_off.p + E;
    a.voff = c->d_off.p + 2 * E;
    a.proff = c->d_off.p + 3 * E;
    a.E = (int)E;
    a.Epad = Epad;
    a.T = nTime;
    a.nW = nW;
    a.a0 = a0;
    a.rho = rhoRef;
    for (int k = 0; k < 3; ++k) a.vinf[k] = (double)hv[k];
    if (f64) {
        CK(nullptr, c->d_rec64.ensure(nrec));
        CK(nullptr, cudaMemsetAsync(c->d_rec64.p, 0, nrec * 8, st));
        a.rec64 = c->d_rec64.p;
    } else {
        CK(nullptr, c->d_rec32.ensure(nrec));
        CK(nullptr, cudaMemsetAsync(c->d_rec32.p, 0, nrec * 4, st));
        a.rec32 = c->d_rec32.p;
        CK(nullptr, c->d_rmax.ensure(1));
        CK(nullptr, cudaMemsetAsync(c->d_rmax.p, 0, sizeof(unsigned), st));
        a.rmax = c->d_rmax.p;
    }
    CK(nullptr, launch_aos_records(a, st));
    // observers in both precisions
    CK(nullptr, c->d_obs64.ensure(3 * (size_t)nObs));
    CK(nullptr, c->d_obs32.ensure(3 * (size_t)nObs));
    std::vector<S> ho(3 * (size_t)nObs);
    CK(nullptr, cudaMemcpyAsync(ho.data(), rObs, ho.size() * sizeof(S), cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaStreamSynchronize(st));
    std::vector<double> o64(ho.size());
    std::vector<float> o32(ho.size());
    for (size_t i = 0; i < ho.size(); ++i) {
        o64[i] = (double)ho[i];
        o32[i] = (float)ho[i];
    }
    CK(nullptr, cudaMemcpyAsync(c->d_obs64.p, o64.data(), o64.size() * 8, cudaMemcpyHostToDevice, st));
    CK(nullptr, cudaMemcpyAsync(c->d_obs32.p, o32.data(), o32.size() * 4, cudaMemcpyHostToDevice, st));
    const double obs_rmin = obs_min_distance(o32.data(), nObs);
    TonalRun r;
    memset(&r, 0, sizeof(r));
    r.g.E = (int)E;
    r.g.Epad = Epad;
    r.g.T = nTime;
    r.g.nW = nW;
    r.g.O = nObs;
    r.g.a0 = a0;
    r.g.rho = rhoRef;
    r.g.oM = oM;
    r.g.dPsi = dPsi;
    r.g.dTau = dTau;
    r.g.lpi = nTime * dPsi;
    for (int q = 0; q < 3; ++q) r.g.vinf[q] = (double)hv[q];
    r.g.obs_rmin = obs_rmin;
    r.precision = f64 ? ACUM_PLAIN_FP64 : ACUM_MIXED;
    r.rmax = f64 ? nullptr : c->d_rmax.p;
    CK(nullptr, plan_tonal(r, 0, 0, 0, c->num_sms, c->smem_optin));
    r.rec = f64 ? (const void*)c->d_rec64.p : (const void*)c->d_rec32.p;
    r.obs64 = c->d_obs64.p;
    r.obs32 = c->d_obs32.p;
    CK(nullptr, c->d_acc.ensure((size_t)nObs * nTime * 2));
    r.acc = c->d_acc.p;
    r.err = c->d_err.p;
    if (r.t.nchunk > 1 || !f64) CK(nullptr, cudaMemsetAsync(c->d_acc.p, 0, (size_t)nObs * nTime * 16, st));
    CK(nullptr, launch_tonal(r, st));
    CK(nullptr, launch_finalize(c->d_acc.p, nObs, nTime, pT, pL, pA, f64 ? 1 : 2, st));
    CK(nullptr, cudaStreamSynchronize(st));
    DeviceErr h;
    CK(nullptr, cudaMemcpy(&h, c->d_err.p, sizeof(h), cudaMemcpyDeviceToHost));
    if (h.bits & ACUM_DEVERR_TIMEOUT) {
        cudaMemset(c->d_err.p, 0, sizeof(DeviceErr));
        return fail(nullptr, ACUM_ERR_TIMEOUT, "a bounded shared-memory pipeline wait ran out");
    }
    return ACUM_OK;
}

}  // namespace

extern "C" int acum_find_pressure_time_history(const float* rObs, const float* tObs, float* pT, float* pL, float* pA,
                                               const float* Xham, const float* Nham, const float* Vham,
                                               const float* PRham, int nSurf, const int* XPtr, const int* NPtr,
                                               const int* VPtr, const int* PRPtr, const int* E, int nObs, int nTime,
                                               float dPsi, float dTau, float a0, float rhoRef, const float* vInf,
                                               float oM, void* stream)
{
    acum::NvtxRange nvtx_range_("acum_find_pressure_time_history");
    return find_pth<float>(rObs, tObs, pT, pL, pA, Xham, Nham, Vham, PRham, nSurf, XPtr, NPtr, VPtr, PRPtr, E, nObs,
                           nTime, dPsi, dTau, a0, rhoRef, vInf, oM, stream);
}

extern "C" int acum_find_pressure_time_history_f64(const double* rObs, const double* tObs, double* pT, double* pL,
                                                   double* pA, const double* Xham, const double* Nham,
                                                   const double* Vham, const double* PRham, int nSurf, const int* XPtr,
                                                   const int* NPtr, const int* VPtr, const int* PRPtr, const int* E,
                                                   int nObs, int nTime, double dPsi, double dTau, double a0,
                                                   double rhoRef, const double* vInf, double oM, void* stream)
{
    acum::NvtxRange nvtx_range_("acum_find_pressure_time_history_f64");
    return find_pth<double>(rObs, tObs, pT, pL, pA, Xham, Nham, Vham, PRham, nSurf, XPtr, NPtr, VPtr, PRPtr, E, nObs,
                            nTime, dPsi, dTau, a0, rhoRef, vInf, oM, stream);
}

extern "C" int acum_preprocess_imper(float* Xham, float* Nham, float* Vham, float* PRham, int nSurf, const int* XPtr,
                                     const int* NPtr, const int* VPtr, const int* PRPtr, const int* E, int nTime,
                                     float dTau, float a0, float rhoRef, float Mref, float CFDscale, int periodic,
                                     int lowpass)
{
    acum::NvtxRange nvtx_range_("acum_preprocess_imper");
    if (!Xham || !Nham || !Vham || !PRham || !XPtr || !NPtr || !VPtr || !PRPtr || !E || nSurf <= 0 || nTime < 4)
        return fail(nullptr, ACUM_ERR_INVALID, "preprocess_imper: bad argument");
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_fail(nullptr, ce, "cudaGetDevice");
    acum_ctx* c = dropin_ctx(dev);
    if (!c) return fail(nullptr, ACUM_ERR_CUDA, "preprocess_imper: cannot create a context");
    // surface rows from the AoS arrays (what read_surf stored, io.cu:318)
    std::vector<int> ne(E, E + nSurf);
    size_t tot = 0;
    for (int i = 0; i < nSurf; ++i) tot += (size_t)nTime * ne[i] * 8;
    std::vector<float> raw(tot);
    size_t off = 0;
    for (int i = 0; i < nSurf; ++i) {
        for (int k = 0; k < nTime; ++k)
            for (int j = 0; j < ne[i]; ++j) {
                float* r = raw.data() + off + ((size_t)k * ne[i] + j) * 8;
                const float* X = Xham + XPtr[i] + (size_t)j * nTime * 4 + (size_t)k * 4;
                const float* N = Nham + NPtr[i] + (size_t)j * nTime * 6 + (size_t)k * 6;
                const float* P = PRham + PRPtr[i] + (size_t)j * nTime * 2 + (size_t)k * 2;
                r[0] = X[0]; r[1] = X[1]; r[2] = X[2]; r[3] = P[0]; r[4] = X[3];
                r[5] = N[0]; r[6] = N[1]; r[7] = N[2];
            }
        off += (size_t)nTime * ne[i] * 8;
    }
    acum_inputs in;
    memset(&in, 0, sizeof(in));
    in.a0 = a0;
    in.rhoRef = rhoRef;
    in.oM = 1.0;
    in.dPsi = 1.0;
    in.Mref = Mref;
    in.CFDscale = CFDscale;
    in.OBSscale = 1.0;
    in.nTime = nTime;
    in.impermeable = 1;
    in.periodic = periodic;
    in.lowpass = lowpass;
    float obs[3] = {1.f, 0.f, 0.f};
    int rc = acum_set_deck(c, &in, 1, obs, nSurf, ne.data(), raw.data(), 0);
    if (rc) return rc;
    c->der.dTau = dTau;  // the caller's step, as preprocess_imper reads it from the global
    std::vector<double> f((size_t)c->E * nTime * kFields);
    rc = acum_get_fields(c, f.data());
    if (rc) return rc;
    long long e = 0;
    for (int i = 0; i < nSurf; ++i)
        for (int j = 0; j < ne[i]; ++j, ++e)
            for (int k = 0; k < nTime; ++k) {
                const double* q = f.data() + ((size_t)e * nTime + k) * kFields;
                float* X = Xham + XPtr[i] + (size_t)j * nTime * 4 + (size_t)k * 4;
                float* N = Nham + NPtr[i] + (size_t)j * nTime * 6 + (size_t)k * 6;
                float* V = Vham + VPtr[i] + (size_t)j * nTime * 6 + (size_t)k * 6;
                float* P = PRham + PRPtr[i] + (size_t)j * nTime * 2 + (size_t)k * 2;
                for (int cc = 0; cc < 4; ++cc) X[cc] = (float)q[cc];
                for (int cc = 0; cc < 6; ++cc) N[cc] = (float)q[4 + cc];
                for (int cc = 0; cc < 6; ++cc) V[cc] = (float)q[10 + cc];
                P[0] = (float)q[16];
                P[1] = (float)q[17];
            }
    return ACUM_OK;
}

namespace {

// The per-element starts of one preprocess_per layout (variables.cu AoS: element j of
// surface i at Ptr[i] + j nTime width) and the extent of each array.
struct PerLayout {
    long long etot = 0;
    std::vector<long long> off;  // [5][etot]: X, N, V, U, PR
    long long extent[5] = {0, 0, 0, 0, 0};
};

int per_layout(int nSurf, const int* XPtr, const int* NPtr, const int* VPtr, const int* UPtr, const int* PRPtr,
               const int* E, int nTime, double dTau, PerLayout& L)
{
    if (!XPtr || !NPtr || !VPtr || !UPtr || !PRPtr || !E || nSurf <= 0 || nTime < 6)
        return fail(nullptr, ACUM_ERR_INVALID, "preprocess_per: bad argument (nTime must be at least 6)");
    if (!(dTau > 0.0) || !std::isfinite(dTau))
        return fail(nullptr, ACUM_ERR_INVALID, "preprocess_per: dTau must be positive and finite");
    if (nTime > acum::kMaxPerSteps)
        return fail(nullptr, ACUM_ERR_UNSUPPORTED, "preprocess_per: more than 4096 steps per period");
    const int width[5] = {4, 6, 6, 6, 4};
    const int* ptr[5] = {XPtr, NPtr, VPtr, UPtr, PRPtr};
    for (int i = 0; i < nSurf; ++i) {
        if (E[i] < 0) return fail(nullptr, ACUM_ERR_INVALID, "preprocess_per: negative element count");
        L.etot += E[i];
    }
    if (L.etot > (1LL << 31) - 1) return fail(nullptr, ACUM_ERR_UNSUPPORTED, "preprocess_per: too many elements");
    L.off.resize((size_t)L.etot * 5);
    long long e = 0;
    for (int i = 0; i < nSurf; ++i)
        for (int j = 0; j < E[i]; ++j, ++e)
            for (int q = 0; q < 5; ++q) {
                if (ptr[q][i] < 0) return fail(nullptr, ACUM_ERR_INVALID, "preprocess_per: negative offset");
                const long long o = (long long)ptr[q][i] + (long long)j * nTime * width[q];
                L.off[(size_t)q * L.etot + e] = o;
                L.extent[q] = std::max(L.extent[q], o + (long long)nTime * width[q]);
            }
    return ACUM_OK;
}

// Enqueues the kernel on `st` over device arrays d[5] (X, N, V, U, PR); the offsets go
// through a stream-ordered allocation.
int per_enqueue(void* const d[5], bool is_double, const PerLayout& L, int nTime, double dTau, double a0,
                double rhoRef, double Mref, double CFDscale, int periodic, int lowpass, cudaStream_t st)
{
    long long* off = nullptr;
    CK(nullptr, cudaMallocAsync((void**)&off, L.off.size() * sizeof(long long), st));
    cudaError_t e = cudaMemcpyAsync(off, L.off.data(), L.off.size() * sizeof(long long), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        acum::PerArgs a;
        memset(&a, 0, sizeof(a));
        a.xoff = off;
        a.noff = off + L.etot;
        a.voff = off + 2 * L.etot;
        a.uoff = off + 3 * L.etot;
        a.proff = off + 4 * L.etot;
        a.E = (int)L.etot;
        a.T = nTime;
        a.two_dt = 2.0 * dTau;
        a.inv_two_dt = 1.0 / a.two_dt;
        a.a0 = a0;
        a.a02 = pow(a0, 2);
        a.rhoRef = rhoRef;
        a.mref2 = pow(Mref, 2);
        a.cfd = CFDscale;
        a.periodic = periodic;
        a.lowpass = lowpass;
        acum::gauss_taps(a.gauss);
        e = acum::launch_per_prep(d[0], d[1], d[2], d[3], d[4], is_double, a, st);
    }
    cudaFreeAsync(off, st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "preprocess_per");
    return ACUM_OK;
}

}  // namespace

// Permeable deck in a context: its rows into the AoS arrays, then preprocess_per on them
// (FP64 storage, so the arrays equal the reference's FP64 build bit for bit).
int acum_ctx::ensure_per_prep()
{
    if (per_ok) return ACUM_OK;
    DeviceGuard g(device);
    if (!d_raw.p) return fail(this, ACUM_ERR_STATE, "no surface rows");
    const int width[5] = {4, 6, 6, 6, 4};
    double* d[5];
    for (int q = 0; q < 5; ++q) {
        CK(this, d_per[q].ensure((size_t)E * T * width[q]));
        d[q] = d_per[q].p;
    }
    CK(this, cudaEventRecord(ev[EV_PREP0], stream));
    CK(this, launch_per_rows(raw_cur ? raw_cur : d_raw.p, d_rawoff.p, d_esurf.p, d_elocal.p, d_ecount.p, (int)E, T, d,
                             stream));
    PerLayout L;
    L.etot = E;
    L.off.resize((size_t)E * 5);
    for (int q = 0; q < 5; ++q)
        for (long long e = 0; e < E; ++e) L.off[(size_t)q * E + e] = e * T * width[q];
    void* dv[5] = {d[0], d[1], d[2], d[3], d[4]};
    int rc = per_enqueue(dv, true, L, T, der.dTau, in.a0, in.rhoRef, in.Mref, in.CFDscale, in.periodic, in.lowpass,
                         stream);
    if (rc) {
        err = g_err;
        return rc;
    }
    CK(this, cudaEventRecord(ev[EV_PREP1], stream));
    launches += 2;
    prep_timed = true;
    per_ok = true;
    return ACUM_OK;
}

extern "C" int acum_get_permeable_fields(acum_ctx* ctx, double* Xham, double* Nham, double* Vham, double* Uham,
                                         double* PRham)
{
    acum::NvtxRange nvtx_range_("acum_get_permeable_fields");
    if (!ctx || !Xham || !Nham || !Vham || !Uham || !PRham) return ACUM_ERR_INVALID;
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "no deck");
    if (!ctx->permeable()) return fail(ctx, ACUM_ERR_STATE, "not a permeable deck (impermeable 1)");
    ctx->begin_run();
    int rc = ctx->ensure_per_prep();
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    double* h[5] = {Xham, Nham, Vham, Uham, PRham};
    const int width[5] = {4, 6, 6, 6, 4};
    for (int q = 0; q < 5; ++q)
        CK(ctx, cudaMemcpyAsync(h[q], ctx->d_per[q].p, (size_t)ctx->E * ctx->T * width[q] * 8, cudaMemcpyDeviceToHost,
                                ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return ACUM_OK;
}

namespace {

// device copies of the caller's five host arrays for one preprocess_per call
struct PerBuffers {
    void* d[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    ~PerBuffers()
    {
        for (void* p : d)
            if (p) cudaFree(p);
    }
};

template <typename S>
int preprocess_per_t(S* Xham, S* Nham, S* Vham, S* Uham, S* PRham, int nSurf, const int* XPtr, const int* NPtr,
                     const int* VPtr, const int* UPtr, const int* PRPtr, const int* E, int nTime, double dTau,
                     double a0, double rhoRef, double Mref, double CFDscale, int periodic, int lowpass)
{
    if (!Xham || !Nham || !Vham || !Uham || !PRham)
        return fail(nullptr, ACUM_ERR_INVALID, "preprocess_per: null array");
    PerLayout L;
    int rc = per_layout(nSurf, XPtr, NPtr, VPtr, UPtr, PRPtr, E, nTime, dTau, L);
    if (rc != ACUM_OK || L.etot == 0) return rc;
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_fail(nullptr, ce, "cudaGetDevice");
    acum_ctx* c = dropin_ctx(dev);
    if (!c) return fail(nullptr, ACUM_ERR_CUDA, "preprocess_per: cannot create a context");
    cudaStream_t st = c->stream;
    S* host[5] = {Xham, Nham, Vham, Uham, PRham};
    PerBuffers b;
    for (int q = 0; q < 5; ++q) {
        CK(nullptr, cudaMalloc(&b.d[q], (size_t)L.extent[q] * sizeof(S)));
        CK(nullptr, cudaMemcpyAsync(b.d[q], host[q], (size_t)L.extent[q] * sizeof(S), cudaMemcpyHostToDevice, st));
    }
    rc = per_enqueue(b.d, sizeof(S) == 8, L, nTime, dTau, a0, rhoRef, Mref, CFDscale, periodic, lowpass, st);
    if (rc != ACUM_OK) return rc;
    c->launches += 1;
    for (int q = 0; q < 5; ++q)
        CK(nullptr, cudaMemcpyAsync(host[q], b.d[q], (size_t)L.extent[q] * sizeof(S), cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaStreamSynchronize(st));
    return ACUM_OK;
}

}  // namespace

extern "C" int acum_preprocess_per(float* Xham, float* Nham, float* Vham, float* Uham, float* PRham, int nSurf,
                                   const int* XPtr, const int* NPtr, const int* VPtr, const int* UPtr,
                                   const int* PRPtr, const int* E, int nTime, float dTau, float a0, float rhoRef,
                                   float Mref, float CFDscale, int periodic, int lowpass)
{
    acum::NvtxRange nvtx_range_("acum_preprocess_per");
    return preprocess_per_t<float>(Xham, Nham, Vham, Uham, PRham, nSurf, XPtr, NPtr, VPtr, UPtr, PRPtr, E, nTime,
                                   dTau, a0, rhoRef, Mref, CFDscale, periodic, lowpass);
}

extern "C" int acum_preprocess_per_f64(double* Xham, double* Nham, double* Vham, double* Uham, double* PRham,
                                       int nSurf, const int* XPtr, const int* NPtr, const int* VPtr,
                                       const int* UPtr, const int* PRPtr, const int* E, int nTime, double dTau,
                                       double a0, double rhoRef, double Mref, double CFDscale, int periodic,
                                       int lowpass)
{
    acum::NvtxRange nvtx_range_("acum_preprocess_per_f64");
    return preprocess_per_t<double>(Xham, Nham, Vham, Uham, PRham, nSurf, XPtr, NPtr, VPtr, UPtr, PRPtr, E, nTime,
                                    dTau, a0, rhoRef, Mref, CFDscale, periodic, lowpass);
}

extern "C" int acum_preprocess_per_device(void* Xham, void* Nham, void* Vham, void* Uham, void* PRham, int is_double,
                                          int nSurf, const int* XPtr, const int* NPtr, const int* VPtr,
                                          const int* UPtr, const int* PRPtr, const int* E, int nTime, double dTau,
                                          double a0, double rhoRef, double Mref, double CFDscale, int periodic,
                                          int lowpass, void* stream)
{
    acum::NvtxRange nvtx_range_("acum_preprocess_per_device");
    if (!Xham || !Nham || !Vham || !Uham || !PRham)
        return fail(nullptr, ACUM_ERR_INVALID, "preprocess_per: null array");
    PerLayout L;
    int rc = per_layout(nSurf, XPtr, NPtr, VPtr, UPtr, PRPtr, E, nTime, dTau, L);
    if (rc != ACUM_OK || L.etot == 0) return rc;
    void* d[5] = {Xham, Nham, Vham, Uham, PRham};
    return per_enqueue(d, is_double != 0, L, nTime, dTau, a0, rhoRef, Mref, CFDscale, periodic, lowpass,
                       (cudaStream_t)stream);
}
