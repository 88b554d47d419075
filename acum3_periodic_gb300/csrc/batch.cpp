// batch.cpp -- many decks on one device, solved by one persistent launch (acum_batch_*).
//
// Each case is an ordinary context (deck upload, GPU preprocessing into the mixed-form
// records) that shares the batch's stream; its surface rows are dropped once the records
// exist.  The batch owns one pool of FP64 bin sums and one pool of pA results, the
// per-case kernel constants, and the work list of the persistent kernel:
//   item = (case, observer tile of W observers, element range)
// with the element range of each case cut so that all items cost about the same
// (total evaluations / (SMs x items_per_sm)), and the list sorted largest first so that
// the blocks' dynamic pick-up ends with the small items (no tail of one big item).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "acum_internal.h"
#include "ctx.h"

using namespace acum;

struct acum_batch {
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    std::vector<acum_ctx*> cases;

    // tile shape and plan: W observers per block, opw per warp, SE elements per stage;
    // rowlen = slots per bin row (the longest whole-row case's nTime, or the ring's)
    int W = 32, SE = 8, opw = 2, ips = 8;
    bool tile_set = false;  // the shape was set (or autotuned); else the default, with fewer
                            // observers per block where its rows do not fit
    bool planned = false;
    int Tmax = 0, rowlen = 0;
    std::vector<int> ring;  // per case: slots of the bin ring its records fit (ring_for), 0 = whole rows
    int nitems = 0;
    std::vector<BatchItem> items;
    std::vector<size_t> acc_off, out_off;
    int fin_tiles = 0;
    DBuf<double> d_acc, d_out;
    DBuf<KParams> d_kp;
    DBuf<BatchItem> d_items;
    DBuf<FinCase> d_fin;
    DBuf<int> d_counter;
    DBuf<DeviceErr> d_err;
    size_t acc_doubles = 0, out_doubles = 0;

    // graph of the persistent run (mode 2)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;

    double last_ms = 0;
    long long last_launches = 0;
    bool have_result = false;
    int last_mode = -1;

    void drop_graph()
    {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
    }
};

namespace {

int bfail(acum_batch* b, int code, const std::string& msg)
{
    if (b) b->err = msg;
    return fail(nullptr, code, msg);
}

int bcuda(acum_batch* b, cudaError_t e, const char* what)
{
    return bfail(b, ACUM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define BK(b, call)                                        \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return bcuda(b, e_, #call); \
    } while (0)

// TonalRun of case c with the batch's tile shape (the fields the kernels read)
TonalRun case_run(const acum_batch* b, const acum_ctx* c, double* acc)
{
    TonalRun r;
    memset(&r, 0, sizeof(r));
    r.g.E = (int)c->E;
    r.g.Epad = c->Epad;
    r.g.T = c->T;
    r.g.nW = c->nW;
    r.g.O = c->nobs;
    r.g.a0 = c->in.a0;
    r.g.rho = c->in.rhoRef;
    r.g.oM = c->der.oM;
    r.g.dPsi = c->der.dPsi;
    r.g.dTau = c->der.dTau;
    r.g.lpi = c->T * c->der.dPsi;
    for (int k = 0; k < 3; ++k) r.g.vinf[k] = c->der.vinf[k];
    r.g.obs_rmin = c->obs_rmin;
    r.precision = ACUM_MIXED;
    r.t.W = b->W;
    r.t.SE = b->SE;
    r.t.NS = batch_stages(b->SE);
    r.t.flush_elems = 512;  // FP32 bin sums over at most 512 elements, as the single-deck plan
    r.t.opw = b->opw;
    r.t.chunk = c->Epad;
    r.t.nchunk = 1;
    r.rec = c->d_rec32.p;
    r.rmax = c->d_rmax.p;
    r.obs32 = c->d_obs32.p;
    r.obs64 = c->d_obs64.p;
    r.acc = acc;
    r.err = b->d_err.p;
    return r;
}

// the work list for a tile shape, largest item first
void build_items(const acum_batch* b, int W, int SE, int ips, std::vector<BatchItem>& out)
{
    out.clear();
    double total = 0;
    for (const acum_ctx* c : b->cases) total += (double)((c->nobs + W - 1) / W) * W * c->Epad * c->T;
    const double target = total / ((double)b->num_sms * ips);
    struct Cost {
        double cost;
        BatchItem it;
    };
    std::vector<Cost> v;
    for (size_t ci = 0; ci < b->cases.size(); ++ci) {
        const acum_ctx* c = b->cases[ci];
        const int tiles = (c->nobs + W - 1) / W;
        const int groups = c->Epad / SE;
        const double per_tile = (double)W * c->Epad * c->T;
        int nchunk = (int)std::ceil(per_tile / std::max(target, 1.0));
        // element chunks of at most ~32 MB of records (as the single-deck plan), so that
        // the items of one chunk, which run close together in time, share it in L2
        const size_t per_elem = (size_t)nwin32(c->T) * kGroups32 * kWin * 4 * sizeof(float);
        const int max_groups = std::max(1, (int)(((size_t)32 << 20) / per_elem) / SE);
        nchunk = std::max(nchunk, (groups + max_groups - 1) / max_groups);
        nchunk = std::max(1, std::min(nchunk, groups));
        const int gpc = (groups + nchunk - 1) / nchunk;
        // chunk-major: equal-cost items of a case stay in this order after the sort
        for (int g0 = 0; g0 < groups; g0 += gpc) {
            const int e0 = g0 * SE, e1 = std::min(groups, g0 + gpc) * SE;
            for (int ot = 0; ot < tiles; ++ot) {
                const int wobs = std::min(W, c->nobs - ot * W);
                v.push_back({(double)wobs * (e1 - e0) * c->T, BatchItem{(int)ci, ot, e0, e1}});
            }
        }
    }
    std::stable_sort(v.begin(), v.end(), [](const Cost& a, const Cost& b2) { return a.cost > b2.cost; });
    out.reserve(v.size());
    for (const Cost& x : v) out.push_back(x.it);
}

bool shape_fits(const acum_batch* b, int W, int SE, int opw)
{
    return batch_smem(W, SE, b->rowlen) + batch_static_smem(SE, opw) <= b->smem_optin;
}

// Which bin ring each case's records fit (from the case's largest |x|, read once), and
// the slots per bin row the batch needs.
int ring_cases(acum_batch* b)
{
    const size_t n = b->cases.size();
    if (b->ring.size() != n) {
        b->ring.assign(n, 0);
        for (size_t i = 0; i < n; ++i) {
            const acum_ctx* c = b->cases[i];
            unsigned bits = 0;
            BK(b, cudaMemcpy(&bits, c->d_rmax.p, sizeof(bits), cudaMemcpyDeviceToHost));
            float r;
            memcpy(&r, &bits, sizeof(r));
            b->ring[i] = ring_for(r, c->der.vinf[0], c->der.vinf[1], c->der.vinf[2], c->in.a0,
                                  c->der.oM / c->der.dPsi, c->obs_rmin, c->T);
        }
    }
    b->Tmax = 0;
    b->rowlen = 0;
    for (size_t i = 0; i < n; ++i) {
        b->Tmax = std::max(b->Tmax, b->cases[i]->T);
        b->rowlen = std::max(b->rowlen, b->ring[i] > 0 ? b->ring[i] : b->cases[i]->T);
    }
    return ACUM_OK;
}

// The default shape (after ring_cases): 32 observers per block, two per warp, 8 elements
// per stage, with as many observers per block as the longest rows leave room for; where
// that leaves fewer than 12 warps of two, one observer per warp if that gives more warps
// (the single-deck wide rings measured likewise).
void default_shape(acum_batch* b)
{
    b->W = 32;
    b->SE = 8;
    b->opw = 2;
    while (b->W > b->opw && !shape_fits(b, b->W, b->SE, b->opw)) b->W -= b->opw;
    if (b->W / 2 < 12) {
        int W1 = 16;
        while (W1 > 1 && !shape_fits(b, W1, b->SE, 1)) --W1;
        if (W1 > b->W / 2 && shape_fits(b, W1, b->SE, 1)) {
            b->W = W1;
            b->opw = 1;
        }
    }
}

int plan(acum_batch* b)
{
    if (b->cases.empty()) return bfail(b, ACUM_ERR_STATE, "the batch has no cases");
    DeviceGuard g(b->device);
    int rc0 = ring_cases(b);
    if (rc0) return rc0;
    if (!b->tile_set) default_shape(b);
    if (!shape_fits(b, b->W, b->SE, b->opw))
        return bfail(b, ACUM_ERR_INVALID, "tile shape does not fit in shared memory for the longest case");
    // pools of sums and results
    const size_t n = b->cases.size();
    b->acc_off.assign(n, 0);
    b->out_off.assign(n, 0);
    size_t acc = 0, out = 0;
    for (size_t i = 0; i < n; ++i) {
        b->acc_off[i] = acc;
        b->out_off[i] = out;
        acc += (size_t)b->cases[i]->nobs * b->cases[i]->T * 2;
        out += (size_t)b->cases[i]->nobs * b->cases[i]->T;
    }
    b->acc_doubles = acc;
    b->out_doubles = out;
    BK(b, b->d_acc.ensure(acc));
    BK(b, b->d_out.ensure(out));
    // per-case constants
    std::vector<KParams> kp(n);
    std::vector<FinCase> fin(n);
    int tiles = 0;
    for (size_t i = 0; i < n; ++i) {
        const acum_ctx* c = b->cases[i];
        TonalRun r = case_run(b, c, b->d_acc.p + b->acc_off[i]);
        fill_kparams(r, kp[i]);
        kp[i].ring = b->ring[i];  // the batched kernel picks the form per case
        kp[i].dual = 0;
        fin[i].acc = b->d_acc.p + b->acc_off[i];
        fin[i].pA = b->d_out.p + b->out_off[i];
        fin[i].O = c->nobs;
        fin[i].T = c->T;
        fin[i].tiles_o = (c->nobs + 31) / 32;
        fin[i].tile0 = tiles;
        tiles += fin[i].tiles_o * ((c->T + 31) / 32);
    }
    b->fin_tiles = tiles;
    build_items(b, b->W, b->SE, b->ips, b->items);
    b->nitems = (int)b->items.size();
    BK(b, b->d_kp.ensure(n));
    BK(b, b->d_fin.ensure(n));
    BK(b, b->d_items.ensure(b->items.size()));
    BK(b, cudaMemcpy(b->d_kp.p, kp.data(), n * sizeof(KParams), cudaMemcpyHostToDevice));
    BK(b, cudaMemcpy(b->d_fin.p, fin.data(), n * sizeof(FinCase), cudaMemcpyHostToDevice));
    BK(b, cudaMemcpy(b->d_items.p, b->items.data(), b->items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
    b->drop_graph();
    b->planned = true;
    return ACUM_OK;
}

// memset of the counter and the sums, the persistent kernel, the finalize
int enqueue_persistent(acum_batch* b, const BatchItem* d_items, int nitems, bool finalize)
{
    BK(b, cudaMemsetAsync(b->d_counter.p, 0, sizeof(int), b->stream));
    BK(b, cudaMemsetAsync(b->d_acc.p, 0, b->acc_doubles * 8, b->stream));
    BK(b, launch_tonal_batch(b->d_kp.p, d_items, nitems, b->d_counter.p, b->W, b->SE, b->opw, b->rowlen,
                             b->num_sms, b->stream));
    if (finalize) BK(b, launch_finalize_batch(b->d_fin.p, (int)b->cases.size(), b->fin_tiles, b->stream));
    return ACUM_OK;
}

int check_err(acum_batch* b)
{
    DeviceErr h;
    BK(b, cudaMemcpy(&h, b->d_err.p, sizeof(h), cudaMemcpyDeviceToHost));
    if (h.bits & ACUM_DEVERR_TIMEOUT) {
        cudaMemset(b->d_err.p, 0, sizeof(DeviceErr));
        return bfail(b, ACUM_ERR_TIMEOUT, "a bounded shared-memory pipeline wait ran out; results are incomplete");
    }
    return ACUM_OK;
}

}  // namespace

extern "C" int acum_batch_create(acum_batch** out, int device)
{
    if (!out) return fail(nullptr, ACUM_ERR_INVALID, "acum_batch_create: null out");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, ACUM_ERR_CUDA, "acum_batch_create: no CUDA device");
    if (device < 0 || device >= ndev) return fail(nullptr, ACUM_ERR_INVALID, "acum_batch_create: bad device index");
    std::unique_ptr<acum_batch> b(new acum_batch());
    b->device = device;
    DeviceGuard g(device);
    BK(nullptr, cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device));
    int optin = 0;
    BK(nullptr, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    b->smem_optin = (size_t)optin;
    BK(nullptr, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    BK(nullptr, cudaEventCreate(&b->ev0));
    BK(nullptr, cudaEventCreate(&b->ev1));
    BK(nullptr, b->d_counter.ensure(1));
    BK(nullptr, b->d_err.ensure(1));
    BK(nullptr, cudaMemset(b->d_err.p, 0, sizeof(DeviceErr)));
    *out = b.release();
    return ACUM_OK;
}

extern "C" int acum_batch_destroy(acum_batch* b)
{
    if (!b) return ACUM_OK;
    {
        DeviceGuard g(b->device);
        cudaStreamSynchronize(b->stream);
        b->drop_graph();
        for (acum_ctx* c : b->cases) acum_destroy(c);
        b->d_acc.release();
        b->d_out.release();
        b->d_kp.release();
        b->d_items.release();
        b->d_fin.release();
        b->d_counter.release();
        b->d_err.release();
        cudaEventDestroy(b->ev0);
        cudaEventDestroy(b->ev1);
        cudaStreamDestroy(b->stream);
    }
    delete b;
    return ACUM_OK;
}

extern "C" const char* acum_batch_last_error(const acum_batch* b) { return b ? b->err.c_str() : ""; }

extern "C" int acum_batch_add(acum_batch* b, const acum_inputs* in, int nobs, const float* obs_file, int nsurf,
                              const int* nelem, const float* raw, int* case_id)
{
    acum::NvtxRange nvtx_range_("acum_batch_add");
    if (!b || !in || !obs_file || !nelem || !raw) return bfail(b, ACUM_ERR_INVALID, "acum_batch_add: null argument");
    if (nsurf <= 0 || nobs <= 0 || in->nTime < 6) return bfail(b, ACUM_ERR_INVALID, "acum_batch_add: bad sizes");
    long long E = 0;
    for (int i = 0; i < nsurf; ++i) {
        if (nelem[i] < 0) return bfail(b, ACUM_ERR_INVALID, "acum_batch_add: negative element count");
        E += nelem[i];
    }
    if (E <= 0) return bfail(b, ACUM_ERR_INVALID, "acum_batch_add: no elements");
    if (in->impermeable == 0)
        return bfail(b, ACUM_ERR_UNSUPPORTED, "acum_batch_add: a permeable deck has no acoustic kernel (main.cu:236)");
    DeviceGuard g(b->device);
    // what the case holds while it is added (rows + records) and afterwards (records,
    // sums, results), against the device's free memory with 1 GiB to spare
    const long long T = in->nTime, nW32 = nwin32((int)T), Epad = (E + 7) / 8 * 8;
    const double rows = (double)E * T * 8 * 4, recs = (double)Epad * nW32 * kGroups32 * kWin * 4 * 4;
    const double sums = (double)nobs * T * 8 * 3;
    size_t free_b = 0, total_b = 0;
    BK(b, cudaMemGetInfo(&free_b, &total_b));
    if (rows + recs + sums + (double)(1ull << 30) > (double)free_b)
        return bfail(b, ACUM_ERR_NOMEM, "acum_batch_add: not enough free device memory for this case");
    acum_ctx* c = nullptr;
    int rc = acum_create(&c, b->device);
    if (rc) return bfail(b, rc, std::string("acum_batch_add: ") + acum_last_global_error());
    cudaStreamDestroy(c->stream);
    c->stream = b->stream;
    c->owns_stream = false;
    rc = acum_set_deck(c, in, nobs, obs_file, nsurf, nelem, raw, 0);
    if (!rc) {
        c->begin_run();
        rc = c->ensure_prep(false, true, false);
    }
    if (!rc && cudaStreamSynchronize(b->stream) != cudaSuccess) rc = cuda_fail(c, cudaGetLastError(), "prep");
    if (rc) {
        std::string m = c->err;
        acum_destroy(c);
        return bfail(b, rc, "acum_batch_add: " + m);
    }
    c->d_raw.release();
    b->cases.push_back(c);
    b->planned = false;
    b->have_result = false;
    b->drop_graph();
    if (case_id) *case_id = (int)b->cases.size() - 1;
    return ACUM_OK;
}

extern "C" int acum_batch_count(const acum_batch* b, int* ncase)
{
    if (!b || !ncase) return ACUM_ERR_INVALID;
    *ncase = (int)b->cases.size();
    return ACUM_OK;
}

extern "C" int acum_batch_prepare(acum_batch* b)
{
    acum::NvtxRange nvtx_range_("acum_batch_prepare");
    if (!b) return ACUM_ERR_INVALID;
    return plan(b);
}

extern "C" int acum_batch_run(acum_batch* b, int precision, int mode)
{
    acum::NvtxRange nvtx_range_("acum_batch_run");
    if (!b) return ACUM_ERR_INVALID;
    if (precision != ACUM_MIXED) return bfail(b, ACUM_ERR_UNSUPPORTED, "batched runs are mixed precision only");
    if (mode < 0 || mode > 2) return bfail(b, ACUM_ERR_INVALID, "mode must be 0, 1 or 2");
    if (!b->planned) {
        int rc = plan(b);
        if (rc) return rc;
    }
    DeviceGuard g(b->device);
    long long launches = 0;
    if (mode == 2 && !b->gexec) {
        BK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_persistent(b, b->d_items.p, b->nitems, true);
        cudaGraph_t gr = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &gr);
        if (rc) {
            if (gr) cudaGraphDestroy(gr);
            return rc;
        }
        BK(b, e);
        b->graph = gr;
        BK(b, cudaGraphInstantiate(&b->gexec, b->graph, 0));
    }
    BK(b, cudaEventRecord(b->ev0, b->stream));
    if (mode == 0) {
        int rc = enqueue_persistent(b, b->d_items.p, b->nitems, true);
        if (rc) return rc;
        launches = 2;
    } else if (mode == 2) {
        BK(b, cudaGraphLaunch(b->gexec, b->stream));
        launches = 2;
    } else {
        for (size_t i = 0; i < b->cases.size(); ++i) {
            acum_ctx* c = b->cases[i];
            c->begin_run();
            int rc = c->run_tonal(ACUM_MIXED, nullptr, nullptr, b->d_out.p + b->out_off[i]);
            if (rc) return bfail(b, rc, "case " + std::to_string(i) + ": " + c->err);
            launches += c->launches;
        }
    }
    BK(b, cudaEventRecord(b->ev1, b->stream));
    BK(b, cudaStreamSynchronize(b->stream));
    float ms = 0;
    BK(b, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    b->last_launches = launches;
    b->last_mode = mode;
    int rc = check_err(b);
    if (mode == 1)
        for (acum_ctx* c : b->cases) {
            int r2 = c->finish_run();
            if (r2 && !rc) rc = bfail(b, r2, c->err);
        }
    if (rc) return rc;
    b->have_result = true;
    return ACUM_OK;
}

extern "C" int acum_batch_result(acum_batch* b, int case_id, double* pA)
{
    if (!b || !pA) return ACUM_ERR_INVALID;
    if (case_id < 0 || case_id >= (int)b->cases.size()) return bfail(b, ACUM_ERR_INVALID, "bad case index");
    if (!b->have_result) return bfail(b, ACUM_ERR_STATE, "no run yet");
    DeviceGuard g(b->device);
    const acum_ctx* c = b->cases[case_id];
    BK(b, cudaMemcpy(pA, b->d_out.p + b->out_off[case_id], (size_t)c->nobs * c->T * 8, cudaMemcpyDeviceToHost));
    return ACUM_OK;
}

extern "C" int acum_batch_timing(const acum_batch* b, double* ms, long long* launches)
{
    if (!b) return ACUM_ERR_INVALID;
    if (ms) *ms = b->last_ms;
    if (launches) *launches = b->last_launches;
    return ACUM_OK;
}

extern "C" int acum_batch_case_timing(const acum_batch* b, int case_id, double* ms)
{
    if (!b || !ms) return ACUM_ERR_INVALID;
    if (case_id < 0 || case_id >= (int)b->cases.size()) return ACUM_ERR_INVALID;
    if (b->last_mode != 1) return ACUM_ERR_STATE;
    return acum_last_timing(b->cases[case_id], 0, ms, nullptr);
}

extern "C" int acum_batch_set_tile(acum_batch* b, int obs_per_block, int elems_per_stage, int items_per_sm)
{
    if (!b) return ACUM_ERR_INVALID;
    if (obs_per_block < 0 || obs_per_block > 16 || items_per_sm < 0 ||
        (elems_per_stage != 0 && elems_per_stage != 2 && elems_per_stage != 4 && elems_per_stage != 8))
        return bfail(b, ACUM_ERR_INVALID, "acum_batch_set_tile: obs_per_block 1..16, elems_per_stage 2, 4 or 8");
    // a kept shape of two observers per warp may hold more observers than 16 warps of one
    b->W = obs_per_block ? obs_per_block : std::min(b->W, 16);
    if (elems_per_stage) b->SE = elems_per_stage;
    if (items_per_sm) b->ips = items_per_sm;
    b->opw = 1;
    b->tile_set = true;
    b->planned = false;
    b->drop_graph();
    return ACUM_OK;
}

extern "C" int acum_batch_set_tile2(acum_batch* b, int obs_per_block, int elems_per_stage, int items_per_sm,
                                    int obs_per_warp)
{
    if (!b) return ACUM_ERR_INVALID;
    if (obs_per_warp != 1 && obs_per_warp != 2)
        return bfail(b, ACUM_ERR_INVALID, "acum_batch_set_tile2: obs_per_warp 1 or 2");
    if (obs_per_warp == 1) return acum_batch_set_tile(b, obs_per_block, elems_per_stage, items_per_sm);
    if (obs_per_block < 0 || obs_per_block > 32 || obs_per_block % 2 != 0 || items_per_sm < 0 ||
        (elems_per_stage != 0 && elems_per_stage != 2 && elems_per_stage != 4 && elems_per_stage != 8))
        return bfail(b, ACUM_ERR_INVALID,
                     "acum_batch_set_tile2: two observers per warp: obs_per_block 2..32 (even), elems_per_stage 2, 4 or 8");
    b->W = obs_per_block ? obs_per_block : 32;
    b->SE = elems_per_stage ? elems_per_stage : 8;
    if (items_per_sm) b->ips = items_per_sm;
    b->opw = 2;
    b->tile_set = true;
    b->planned = false;
    b->drop_graph();
    return ACUM_OK;
}

extern "C" int acum_batch_get_tile(const acum_batch* b, int* obs_per_block, int* elems_per_stage, int* items_per_sm)
{
    if (!b) return ACUM_ERR_INVALID;
    if (obs_per_block) *obs_per_block = b->W;
    if (elems_per_stage) *elems_per_stage = b->SE;
    if (items_per_sm) *items_per_sm = b->ips;
    return ACUM_OK;
}

extern "C" int acum_batch_get_obs_per_warp(const acum_batch* b, int* obs_per_warp)
{
    if (!b || !obs_per_warp) return ACUM_ERR_INVALID;
    *obs_per_warp = b->opw;
    return ACUM_OK;
}

namespace {

// A probe work list: items of `chunk` elements (every observer tile of every case), every
// k-th of them so that about `target` items remain.  Returns the evaluations it holds.
double probe_items(const acum_batch* b, int W, int SE, int chunk, long target, std::vector<BatchItem>& out)
{
    std::vector<BatchItem> all;
    std::vector<double> cost;
    for (size_t ci = 0; ci < b->cases.size(); ++ci) {
        const acum_ctx* c = b->cases[ci];
        const int tiles = (c->nobs + W - 1) / W;
        for (int e0 = 0; e0 < c->Epad; e0 += chunk)
            for (int ot = 0; ot < tiles; ++ot) {
                const int e1 = std::min(c->Epad, e0 + chunk) / SE * SE;
                if (e1 <= e0) continue;
                all.push_back(BatchItem{(int)ci, ot, e0, e1});
                cost.push_back((double)std::min(W, c->nobs - ot * W) * (e1 - e0) * c->T);
            }
    }
    const size_t k = std::max<size_t>(1, all.size() / (size_t)std::max<long>(1, target));
    out.clear();
    double ev = 0;
    for (size_t i = 0; i < all.size(); i += k) {
        out.push_back(all[i]);
        ev += cost[i];
    }
    return ev;
}

// device time of one persistent launch over `items` (the second of two launches)
int time_items(acum_batch* b, DBuf<BatchItem>& d, const std::vector<BatchItem>& items, double* ms)
{
    BK(b, d.ensure(items.size()));
    BK(b, cudaMemcpy(d.p, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
    float f = 0;
    for (int rep = 0; rep < 2; ++rep) {
        BK(b, cudaEventRecord(b->ev0, b->stream));
        int rc = enqueue_persistent(b, d.p, (int)items.size(), false);
        if (rc) return rc;
        BK(b, cudaEventRecord(b->ev1, b->stream));
        BK(b, cudaStreamSynchronize(b->stream));
        BK(b, cudaEventElapsedTime(&f, b->ev0, b->ev1));
    }
    *ms = f;
    return check_err(b);
}

// Greedy list scheduling of the work list (largest first) on `slots` blocks that each
// take the next item when they finish one: the predicted makespan in ms.
double makespan(const acum_batch* b, const std::vector<BatchItem>& items, int W, int slots, double ms_per_eval,
                double ms_per_item)
{
    std::vector<double> heap(slots, 0.0);  // min-heap of block finish times
    auto cmp = [](double x, double y) { return x > y; };
    std::make_heap(heap.begin(), heap.end(), cmp);
    double end = 0;
    for (const BatchItem& it : items) {
        const acum_ctx* c = b->cases[it.c];
        const double ev = (double)std::min(W, c->nobs - it.ot * W) * (it.e1 - it.e0) * c->T;
        std::pop_heap(heap.begin(), heap.end(), cmp);
        const double t = heap.back() + ms_per_item + ev * ms_per_eval;
        heap.back() = t;
        std::push_heap(heap.begin(), heap.end(), cmp);
        end = std::max(end, t);
    }
    return end;
}

}  // namespace

extern "C" int acum_batch_autotune(acum_batch* b, int probe_per_sm, double* best_ms)
{
    acum::NvtxRange nvtx_range_("acum_batch_autotune");
    if (!b) return ACUM_ERR_INVALID;
    if (b->cases.empty()) return bfail(b, ACUM_ERR_STATE, "the batch has no cases");
    if (probe_per_sm < 0) return bfail(b, ACUM_ERR_INVALID, "probe_per_sm must be >= 0");
    const int per_sm = probe_per_sm > 0 ? probe_per_sm : 8;
    DeviceGuard g(b->device);
    int rc0 = ring_cases(b);
    if (rc0) return rc0;
    const long target = (long)per_sm * b->num_sms;
    // 1. kernel throughput of every (observers per block, elements per stage): one
    //    persistent launch over a spread of 128-element items from all cases (items of
    //    the size real work lists use: with 32-element items the per-item start-up and
    //    ring fill weigh on the deeper stages and the probe favoured 4 elements per
    //    stage where 8 are faster)
    //    (one observer per warp: 8, 12, 16 observers per block x 2, 4, 8 elements per stage;
    //    two: 16, 24, 32 x 2, 4, 8)
    struct Shape {
        int W, SE, opw;
    };
    std::vector<Shape> shapes;
    for (int W : {8, 12, 16})
        for (int SE : {2, 4, 8}) shapes.push_back({W, SE, 1});
    for (int W : {16, 24, 32})
        for (int SE : {2, 4, 8}) shapes.push_back({W, SE, 2});
    double best_rate = 0;
    default_shape(b);  // kept when no probed shape fits the longest rows
    int bw = b->W, bse = b->SE, bopw = b->opw;
    b->tile_set = true;  // plan() keeps each probed shape
    DBuf<BatchItem> d_probe;
    std::vector<BatchItem> probe;
    for (const Shape& sh : shapes) {
        if (!shape_fits(b, sh.W, sh.SE, sh.opw)) continue;
        b->W = sh.W;
        b->SE = sh.SE;
        b->opw = sh.opw;
        int rc = plan(b);
        if (rc) return rc;
        const double ev = probe_items(b, sh.W, sh.SE, 128, target, probe);
        double ms = 0;
        rc = time_items(b, d_probe, probe, &ms);
        if (rc) return rc;
        const double rate = ev / std::max(ms, 1e-6);
        if (rate > best_rate) {
            best_rate = rate;
            bw = sh.W;
            bse = sh.SE;
            bopw = sh.opw;
        }
    }
    // 2. for the fastest shape, the per-item and per-evaluation costs from two probes of
    //    different item sizes, then items per SM by the predicted makespan of the
    //    largest-first dynamic schedule
    b->W = bw;
    b->SE = bse;
    b->opw = bopw;
    b->tile_set = true;
    int rc = plan(b);
    if (rc) return rc;
    double ev1 = probe_items(b, bw, bse, 64, target, probe), ms1 = 0;
    const double n1 = (double)probe.size();
    rc = time_items(b, d_probe, probe, &ms1);
    if (rc) return rc;
    double ev2 = probe_items(b, bw, bse, 256, target, probe), ms2 = 0;
    const double n2 = (double)probe.size();
    rc = time_items(b, d_probe, probe, &ms2);
    if (rc) return rc;
    d_probe.release();
    const int slots = b->num_sms * batch_blocks_per_sm(bw, bse, bopw, b->rowlen);
    // ms = (n ov + ev c) / slots for a launch whose items spread over all slots
    double c_ev = 0, ov = 0;
    const double det = n1 * ev2 - n2 * ev1;
    if (std::fabs(det) > 0) {
        ov = (ms1 * ev2 - ms2 * ev1) / det * slots;
        c_ev = (n1 * ms2 - n2 * ms1) / det * slots;
    }
    if (!(c_ev > 0) || !(ov >= 0)) {  // noisy probes: per-evaluation cost only
        c_ev = ms2 * slots / std::max(ev2, 1.0);
        ov = 0;
    }
    double best = 1e300;
    int bips = b->ips;
    for (int ips : {4, 8, 16, 32}) {
        b->ips = ips;
        std::vector<BatchItem> items;
        build_items(b, bw, bse, ips, items);
        const double t = makespan(b, items, bw, slots, c_ev, ov);
        if (t < best) {
            best = t;
            bips = ips;
        }
    }
    b->ips = bips;
    rc = plan(b);
    if (rc) return rc;
    b->have_result = false;
    if (best_ms) *best_ms = best;
    return ACUM_OK;
}
