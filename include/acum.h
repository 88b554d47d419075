/*
 * acum.h -- C ABI of the GB300-native ACUM-3 periodic acoustic path.
 *
 * Two families of entry points:
 *
 *  1. Reference-shaped drop-ins.  Same arguments, same meaning and the same accumulate
 *     semantics as the two hot-path calls of the reference driver, so a maintainer can
 *     swap them in at main.cu:236 and main.cu:150 with no other change:
 *       acum_find_pressure_time_history      replaces core.cu:18 (launched at main.cu:236)
 *       acum_find_pressure_time_history_f64  the same call on the FP64 build's arrays
 *       acum_find_bb_noise                   replaces bb_core.cu:11 (called at main.cu:150)
 *       acum_preprocess_imper                replaces preprocess.cu:228 on caller arrays
 *       acum_preprocess_per(_f64)            replaces preprocess.cu:8 (main.cu:87, permeable)
 *
 *  2. A context API that owns the deck on the device and runs the whole path: the file
 *     readers and writers keep the reference's formats (io.cu), preprocessing and all
 *     compute run on the GPU, and the adjoint and batched forms are reachable here.
 *
 * Conventions: every call returns int status (ACUM_OK = 0, negative = error class) and
 * never exits the process; acum_last_error() gives the message of the last failure of a
 * context, acum_last_global_error() that of a context-free call.  Pointers documented as
 * "device" must be CUDA device (or managed) memory of the context's device; "host"
 * pointers are ordinary or pinned host memory.  All arrays are dense, C order.  A
 * context is used by one host thread at a time; different contexts are independent.
 */
#ifndef ACUM_H
#define ACUM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ACUM_OK 0
#define ACUM_ERR_INVALID (-1)     /* bad argument or inconsistent sizes */
#define ACUM_ERR_IO (-2)          /* deck file missing or malformed */
#define ACUM_ERR_CUDA (-3)        /* CUDA runtime error (message has the CUDA error) */
#define ACUM_ERR_NOMEM (-4)       /* device or host allocation failed */
#define ACUM_ERR_STATE (-5)       /* call out of order (e.g. a run before a deck) */
#define ACUM_ERR_TIMEOUT (-6)     /* a bounded device wait ran out; the context stays usable */
#define ACUM_ERR_GEOMETRY (-7)    /* invalid geometry met on the device (see error word) */
#define ACUM_ERR_UNSUPPORTED (-8) /* option outside what the library implements */

/* precision of the tonal forms */
#define ACUM_PLAIN_FP64 0 /* FP64 end to end; matches the reference's FP64 build */
#define ACUM_MIXED 1      /* FP32 integrand, FP64-anchored observer time, FP32 bins summed in FP64 */

/* bits of the device error word (acum_device_error_word) */
#define ACUM_DEVERR_DISC 0x1u       /* negative discriminant in the retarded-time solve */
#define ACUM_DEVERR_ORDER 0x2u      /* observer time not increasing between steps (|Mr| >= 1) */
#define ACUM_DEVERR_NONFINITE 0x4u  /* non-finite integrand */
#define ACUM_DEVERR_TIMEOUT 0x8u    /* a bounded shared-memory pipeline wait ran out */

typedef struct acum_ctx acum_ctx;

/* ---------------------------------------------------------------- context */

int acum_create(acum_ctx** out, int device);
int acum_destroy(acum_ctx* ctx);
const char* acum_last_error(const acum_ctx* ctx);
const char* acum_last_global_error(void);
int acum_version(void);

/* The `input` file's settings (io.cu:12-101).  Angles in degrees, as in the file. */
typedef struct {
    double a0, rhoRef, pRef, oM, dPsi, Minf, Mref, xy_angle, xz_angle, CFDscale, OBSscale;
    int nTime, impermeable, periodic, lowpass, BB_noise;
} acum_inputs;

/* Reads input, obs.dat, surfaces/surface_*.dat (and input_BB, BB_inputs/ when
 * BB_noise = 1) from `dir` with the semantics of io.cu (read_inputs, read_observers,
 * read_surf, read_BB_inputs).  Replaces any deck already in the context. */
int acum_load_deck(acum_ctx* ctx, const char* dir);

/* The same deck from memory.  `obs_file` [nobs][3] are obs.dat values (OBSscale is
 * applied as read_observers does); `raw` holds the surface_*.dat rows of all surfaces,
 * surface after surface, each [nTime][nelem[i]][ncol]: ncol = 8, x,y,z,Cp,A,nx,ny,nz, for
 * impermeable decks (io.cu:321), ncol = 12, x,y,z,u,v,w,P,rho,ds,nx,ny,nz, for permeable
 * ones (in->impermeable = 0, io.cu:286).  The arrays are copied; `raw` may be pinned host
 * memory or device memory (raw_on_device = 1).
 *
 * Permeable decks follow main.cu: acum_preprocess runs preprocess_per (main.cu:87) on the
 * GPU, the tonal calls return pT = pL = pA = 0 (main.cu:236 launches no kernel for them;
 * main.cu:123-130 zeroed the arrays), acum_write_outputs writes those zero files, and the
 * broadband path is unaffected; the impermeable-only calls (fields, adjoint, batches)
 * return ACUM_ERR_UNSUPPORTED.  At most 4096 steps per period. */
int acum_set_deck(acum_ctx* ctx, const acum_inputs* in, int nobs, const float* obs_file, int nsurf,
                  const int* nelem, const float* raw, int raw_on_device);

/* Replaces only the surface rows (same sizes as the deck), e.g. for a new flight state;
 * host or device memory.  Marks the deck for re-preprocessing. */
int acum_update_surfaces(acum_ctx* ctx, const float* raw, int raw_on_device);

/* A permeable deck's arrays after preprocess_per (preprocess.cu:8-226, main.cu:87), in
 * the reference's AoS layout (variables.cu:54, elements surface after surface, each
 * [nTime][width]): Xham [E][nTime][4] = x,y,z,ds; Nham [6] = n, ndot; Vham [6] = V, Vdot;
 * Uham [6] = u, udot; PRham [4] = P, Pdot, rho, rhodot.  FP64, equal bit for bit to the
 * reference's FP64 build on the same rows; host memory.  ACUM_ERR_STATE for an
 * impermeable deck. */
int acum_get_permeable_fields(acum_ctx* ctx, double* Xham, double* Nham, double* Vham, double* Uham,
                              double* PRham);

/* Broadband inputs from memory (read_BB_inputs layout, io.cu:337-700).  Per BB surface
 * i: span, omega, ccw, psi_offset, trip, rotate[3], translate[3]; nsect[i] sections with
 * geom [nsect][4] = r/R, y/R, z/R, c/R and data [nTime][nsect][7] = BLT_s, BLT_p, DT_s,
 * DT_p, cn, cc, theta as in the file (cn, cc are divided by (r/R)^2 here when omega != 0,
 * as the reader does); tables of sizes ns_t, na_t, nm_t, nr_t with axes sect/aoa/mach/re
 * and data [ns_t][nm_t][nr_t][na_t][7] = cl, cd, cm, bl_u, bl_l, disp_u, disp_l.  All
 * per-surface arrays are concatenated surface after surface. */
typedef struct {
    int nsurf, t_del;
    const double *span, *omega, *psi_offset, *rotate, *translate;
    const int *ccw, *trip, *nsect;
    const float *geom, *data;
    const int *ns_t, *na_t, *nm_t, *nr_t;
    const float *sect_t, *aoa_t, *mach_t, *re_t, *table;
} acum_bb_desc;
int acum_set_bb(acum_ctx* ctx, const acum_bb_desc* bb);

/* sizes: out[0]=nSurf, [1]=nTime, [2]=nObs, [3]=elements, [4]=BB sections, [5]=BB_noise */
/* Writes surfaces/surfaces.acumbin in a deck directory: the surface rows as read from the
 * text files (io.cu:206-333), with the size and modification time of each text file.
 * acum_load_deck and acum_read_deck_sizes then read the rows from it instead of parsing
 * the text while no text file has changed; a stale or foreign cache is ignored.  Host
 * only.  (No reference counterpart.) */
int acum_write_surface_cache(const char* dir);

/* Parses and validates a deck directory on the host only (no device needed): the same
 * readers and checks as acum_load_deck.  out[6] as acum_get_sizes. */
int acum_read_deck_sizes(const char* dir, long long* out);
int acum_get_sizes(const acum_ctx* ctx, long long* out);

/* Uploads what is not on the device yet and runs preprocess_imper's steps on the GPU
 * (scaling, make_periodic, optional lowpass, d/dtau), building both record layouts. */
int acum_preprocess(acum_ctx* ctx);

/* Copies the preprocessed per-element-step fields back, [elements][nTime][18] =
 * x,y,z,ds, n(3), ndot(3), V(3), Vdot(3), P, Pdot (the contents of Xham/Nham/Vham/PRham). */
int acum_get_fields(acum_ctx* ctx, double* host_fields);

/* Tonal noise.  Outputs [nTime][nObs] (main.cu:123-130 layout), overwritten, host memory;
 * any of pT/pL/pA may be NULL.  Preprocesses first if needed. */
int acum_tonal(acum_ctx* ctx, int precision, double* pT, double* pL, double* pA);

/* The whole tonal path from host buffers in one call: copies `raw` (same layout as
 * acum_set_deck, host memory, pinned for full speed) to the device, preprocesses, runs
 * the kernels and copies pA [nTime][nObs] back.  The deck's sizes must not change. */
int acum_tonal_from_host(acum_ctx* ctx, int precision, const float* raw, double* pA_host);

/* Tonal with device outputs [nTime][nObs], on the context stream; no host sync.  With
 * all three pointers NULL the results stay in the context's own device buffer. */
int acum_tonal_device(acum_ctx* ctx, int precision, double* d_pT, double* d_pL, double* d_pA);

/* Device address of the context's copy of the surface rows (acum_set_deck layout), so a
 * solver on the same GPU can write new rows in place; call acum_mark_surfaces_changed
 * afterwards so the next run preprocesses them again. */
int acum_surfaces_device_ptr(acum_ctx* ctx, float** p);
int acum_mark_surfaces_changed(acum_ctx* ctx);

/* Waits for the context's streams (all runs issued so far) and reports a device timeout
 * of any of them (ACUM_ERR_TIMEOUT). */
int acum_sync(acum_ctx* ctx);
/* acum_tonal_from_host without waiting: the host rows (acum_set_deck layout, pinned
 * memory for the copy to overlap) are copied into one of two device row buffers on a copy
 * stream while the previous call's solve runs (two buffers besides the context's own
 * rows), then preprocessed and solved; pA
 * [nTime][nObs] is written to pA_host when the solve ends.  Returns at once; acum_sync
 * waits.  raw and pA_host must stay valid until then.  The context's own rows (the last
 * acum_set_deck / acum_update_surfaces) stay in place; acum_tonal runs on those. */
int acum_tonal_from_host_async(acum_ctx* ctx, int precision, const float* raw, double* pA_host);
/* The context's CUDA stream (a cudaStream_t), on which every run of the context is
 * issued; a caller may record events on it or order its own work after it. */
int acum_stream(acum_ctx* ctx, void** stream);

/* Broadband: BBspl [nObs][42][7] and BBoaspl [nObs] in dB (bb_core.cu:563-583 layout),
 * host memory, overwritten (the -100 dB seeding of main.cu:132-142 is applied inside).
 * aa_mode selects the convected emission time of bb_core.cu:517-520: 0 uses
 * aa = a0^2 - |vInf|^2 (the formula's intent), 1 uses aa = 0 (the value the reference's
 * uninitialised variable takes in a zero-initialising build). */
int acum_bpm(acum_ctx* ctx, int aa_mode, double* BBspl, double* BBoaspl);

/* Writes pT.out, pL.out, pA.out (io.cu:137-203) and, if broadband was run,
 * bb_oaspl.out and bb_spl.dat (io.cu:702-796) into `dir`, byte-format compatible. */
int acum_write_outputs(acum_ctx* ctx, const char* dir);

/* Adjoint of J = sum_obs mean_bins(pA^2) with respect to the surface rows: gradients
 * [elements][nTime] for Cp, [elements][nTime][3] for positions and normals (file
 * coordinates, before CFDscale), host memory.  J is returned in *J.  Requires
 * lowpass = 0.  dJ_dpA may be NULL (the objective above) or [nTime][nObs] host. */
int acum_tonal_adjoint(acum_ctx* ctx, int precision, const double* dJ_dpA, double* J, double* g_cp, double* g_x,
                       double* g_n);

/* Device error word (ACUM_DEVERR_* bits) accumulated since the last reset. */
int acum_device_error_word(acum_ctx* ctx, uint32_t* out, int reset);

/* Timing of the last run's kernels, measured with CUDA events on the launching stream:
 * which = 0 tonal kernel, 1 preprocess, 2 finalize, 3 bpm (its six kernels), 4 adjoint,
 * 5 whole call, 6 the broadband observer contraction alone (bb_obs_kernel).
 * *launches is the number of kernel launches of this library in the last run. */
int acum_last_timing(const acum_ctx* ctx, int which, double* ms, long long* launches);

/* Tile shape of the tonal kernels (0 = let the library choose): observers per block
 * (1..16; the mixed ring kernel with two observers per warp 1..32), elements per pipeline
 * stage (mixed form: 2, 4 or 8; 2 or 4 with two observers per warp) and work items per
 * SM. */
int acum_set_tile(acum_ctx* ctx, int obs_per_block, int elems_per_stage, int items_per_sm);
/* Observers evaluated per warp of the mixed tonal ring kernel on the records it loads
 * once: 1 or 2 (0 = let the library choose; the whole-row kernel evaluates one). */
int acum_set_obs_per_warp(acum_ctx* ctx, int obs_per_warp);
/* Record stages of the mixed tonal kernel (whole rows, one observer per warp) copied once
 * into tensor memory and read from there by every warp, instead of read by every warp
 * from shared memory: 1 = yes, 2 = no, 0 = let the library choose. */
int acum_set_tensor_memory(acum_ctx* ctx, int use);
/* Bins of the mixed tonal kernel: 0 = a sliding ring of bins per observer (the ring
 * kernel, 512 slots), with wide-ring kernels (1024 slots in decks of more than 1024 steps,
 * 2048 slots in decks of more than 2048) and the whole-row kernel launched behind it, each
 * for records whose retarded times spread too far for the rings before it (the default);
 * 1 = whole rows of the period only. */
int acum_set_ring(acum_ctx* ctx, int mode);
/* The ring side of the last tonal plan (out holds 11 ints): out[0] ring slots per
 * observer (0: whole rows only), [1] observers per block, [2] elements per stage and [3]
 * pipeline stages of the whole-row kernel behind the ring kernels, [4] the slots of the
 * ring whose kernel did the work (0: the whole-row kernel; synchronises the context's
 * stream), [5] slots of the 1024-slot wide ring (0: not planned), [6] observers per block
 * and [7] pipeline stages of its kernel, [8], [9], [10] the same for the 2048-slot one. */
int acum_last_plan_ring(acum_ctx* ctx, int* out);
/* The plan of the last tonal run (out holds 8 ints): out[0] observers per block,
 * [1] elements per stage, [2] pipeline stages, [3] elements per work item, [4] element
 * chunks, [5] work items, [6] observers per warp, [7] 1 if the record stages were read
 * from tensor memory. */
int acum_last_plan(const acum_ctx* ctx, int* out);

/* Self-test of the bounded wait that every pipelined kernel uses on its barriers: one
 * block waits on a barrier that is completed (arrive = 1) or never completed (arrive = 0)
 * and gives up after limit_s (0 < limit_s <= 10); *timed_out = 1 if it gave up, *waited_s
 * the device time it waited.  The kernels themselves give up after 2 s, record
 * ACUM_DEVERR_TIMEOUT and return; the context stays usable. */
int acum_selftest_wait(int device, double limit_s, int arrive, int* timed_out, double* waited_s);
/* Self-test of the tensor-memory path of the record stages: a known pattern laid out as
 * one element-pair tile is copied from shared memory into tensor memory and read back by
 * every warp of a block.  *mismatches = words that differ (0 = pass; -1 = the copy did not
 * complete within the bounded wait); readback (optional, 4 x 32 x 40 words) = what warps
 * 0-3 read, lane by lane. */
int acum_selftest_tmem(int device, int* mismatches, unsigned* readback);

/* Measured FMA throughput of `device` in TFLOP/s: which = 0 FP32, 1 FP64 (a short
 * FMA-chain kernel timed with CUDA events; the CUDA-core peaks of the roofline). */
int acum_measure_peak(int device, int which, double* tflops);

/* Pinned host memory for staging (cudaHostAlloc); free with acum_host_free. */
int acum_host_alloc(void** p, size_t bytes);
int acum_host_free(void* p);

/* ------------------------------------------------- reference-shaped drop-ins */

/* Replaces findPressureTimeHistory (core.cu:18) as launched at main.cu:236: the same
 * arguments, all device pointers, FP32 storage; accumulates into pT, pL, pA [nTime][nObs].
 * The arrays are those preprocess_imper produced (AoS Xham/Nham/Vham/PRham with the
 * XPtr/NPtr/VPtr/PRPtr offsets and E[] counts, all in device memory as the reference
 * passes them).  Runs the mixed-precision kernel; `stream` may be NULL (default stream).
 * Synchronises the stream before returning. */
int acum_find_pressure_time_history(const float* rObs, const float* tObs, float* pT, float* pL, float* pA,
                                    const float* Xham, const float* Nham, const float* Vham, const float* PRham,
                                    int nSurf, const int* XPtr, const int* NPtr, const int* VPtr, const int* PRPtr,
                                    const int* E, int nObs, int nTime, float dPsi, float dTau, float a0,
                                    float rhoRef, const float* vInf, float oM, void* stream);

/* The same call on the FP64 build's arrays (every `float` of core.cu:18 a `double`);
 * runs the plain FP64 kernel. */
int acum_find_pressure_time_history_f64(const double* rObs, const double* tObs, double* pT, double* pL,
                                        double* pA, const double* Xham, const double* Nham, const double* Vham,
                                        const double* PRham, int nSurf, const int* XPtr, const int* NPtr,
                                        const int* VPtr, const int* PRPtr, const int* E, int nObs, int nTime,
                                        double dPsi, double dTau, double a0, double rhoRef, const double* vInf,
                                        double oM, void* stream);

/* The same call as acum_find_pressure_time_history for callers that cannot allocate
 * device memory (no counterpart in the reference): a solver or plugin host that has given
 * all device memory to its own pool and forbids allocations outside it, or a latency-bound
 * loop that cannot afford cudaMalloc/cudaFree, which synchronise the whole device.  It
 * allocates nothing -- no cudaMalloc, no host heap -- and uses a fixed 128 MiB scratch
 * array in device memory that every GPU loading this library holds until exit.  Limit:
 * records (64 B per element and record slot: elements rounded up to 8, ceil(nTime / 31)
 * windows of 32 slots) plus 16 B per observer-step must fit in 128 MiB, else
 * ACUM_ERR_INVALID (acum_noalloc_last_error()
 * gives the sizes); at most 256 surfaces.  Otherwise it accepts and refuses the inputs the
 * allocating call does (nTime >= 4; tObs[t] = t*dPsi, as main.cu:124 builds it, else
 * ACUM_ERR_UNSUPPORTED).  The first call on a device looks up the scratch address (with
 * that device current); make that first call before any stream capture.  Every call
 * synchronises `stream` before it returns.  All calls share the scratch: calls whose GPU
 * work overlaps race, so serialise them.  acum_noalloc_last_error() is per host thread. */
int acum_find_pressure_time_history_noalloc(const float* rObs, const float* tObs, float* pT, float* pL, float* pA,
                                            const float* Xham, const float* Nham, const float* Vham,
                                            const float* PRham, int nSurf, const int* XPtr, const int* NPtr,
                                            const int* VPtr, const int* PRPtr, const int* E, int nObs, int nTime,
                                            float dPsi, float dTau, float a0, float rhoRef, const float* vInf,
                                            float oM, void* stream);
const char* acum_noalloc_last_error(void);

/* Replaces preprocess_imper (preprocess.cu:228) on caller arrays: host AoS Xham [etot*
 * nTime*4], Nham [*6], Vham [*6], PRham [*2] laid out with the reference's XPtr/NPtr/
 * VPtr/PRPtr offsets (E[] counts, host); updated in place with the same meaning. */
int acum_preprocess_imper(float* Xham, float* Nham, float* Vham, float* PRham, int nSurf, const int* XPtr,
                          const int* NPtr, const int* VPtr, const int* PRPtr, const int* E, int nTime, float dTau,
                          float a0, float rhoRef, float Mref, float CFDscale, int periodic, int lowpass);

/* Replaces preprocess_per (preprocess.cu:8, called at main.cu:87 when impermeable = 0) on
 * caller arrays: host AoS Xham [*4] (x, y, z, ds), Nham [*6] (n, ndot), Vham [*6] (V,
 * Vdot), Uham [*6] (u, udot), PRham [*4] (P, Pdot, rho, rhodot), element j of surface i
 * at Ptr[i] + j*nTime*width as the reference lays them out (variables.cu:11-42, E[]
 * counts, host).  Updated in place with the same meaning: x, ds, u, rho, P scaled; u, rho,
 * P low-passed when lowpass = 1; their derivatives periodic (periodic = 1) or end-biased;
 * ndot, V, Vdot periodic.  The GPU computes in FP64 in the reference's order of
 * operations: the _f64 form (the FP64 build's arrays) equals that build bit for bit, the
 * float form gives those results rounded once to float.  6 <= nTime <= 4096 (the 13-tap
 * filter's periodic index wraps once, the biased ends read du[3]): ACUM_ERR_INVALID
 * below, ACUM_ERR_UNSUPPORTED above. */
int acum_preprocess_per(float* Xham, float* Nham, float* Vham, float* Uham, float* PRham, int nSurf, const int* XPtr,
                        const int* NPtr, const int* VPtr, const int* UPtr, const int* PRPtr, const int* E, int nTime,
                        float dTau, float a0, float rhoRef, float Mref, float CFDscale, int periodic, int lowpass);
int acum_preprocess_per_f64(double* Xham, double* Nham, double* Vham, double* Uham, double* PRham, int nSurf,
                            const int* XPtr, const int* NPtr, const int* VPtr, const int* UPtr, const int* PRPtr,
                            const int* E, int nTime, double dTau, double a0, double rhoRef, double Mref,
                            double CFDscale, int periodic, int lowpass);
/* The same on arrays already in device memory (float, or double when is_double = 1), for
 * a caller whose surface data is on the GPU; XPtr ... PRPtr and E are host arrays.  Work
 * is enqueued on `stream` (NULL = the default stream) and the call returns without
 * waiting for it. */
int acum_preprocess_per_device(void* Xham, void* Nham, void* Vham, void* Uham, void* PRham, int is_double, int nSurf,
                               const int* XPtr, const int* NPtr, const int* VPtr, const int* UPtr, const int* PRPtr,
                               const int* E, int nTime, double dTau, double a0, double rhoRef, double Mref,
                               double CFDscale, int periodic, int lowpass, void* stream);

/* Replaces findBBnoise (bb_core.cu:11) as called at main.cu:150: the same 39 arguments,
 * host pointers, FP32 storage; BBspl [nObs][nf2][7] and BBoaspl [nObs] are updated as the
 * reference does (they arrive seeded, normally with -100 dB).  Computes on the GPU with
 * aa_mode 0 (see acum_bpm). */
int acum_find_bb_noise(int nSurf_BB, int nObs, int nTime, float dTau, const float* span, const float* omega,
                       const int* ccw, const float* psi_offset, const int* trip, const float* rotate,
                       const float* translate, const int* xsPtr, const int* dsPtr, const int* nsect,
                       const float* xyzcR, const float* bbdata, const int* nsect_t, const int* nmach_t,
                       const int* naoa_t, const int* nre_t, const int* aPtr, const int* mPtr, const int* rPtr,
                       const int* sPtr, const int* dPtr, const float* sect_t, const float* mach_t, const float* aoa_t,
                       const float* re_t, const float* bbdata_t, int t_del, const float* vInf, const float* rObs,
                       const float* tObs, int nf2, const float* ff, float a0, float* BBspl, float* BBoaspl);

/* --------------------------------------------------------------- batching */

/* No reference counterpart: the reference solves one deck per process (main.cu).  A batch
 * holds many independent decks ("cases") resident on one device and runs all their tonal
 * solves (mixed precision) in one persistent launch: one block per SM takes work items
 * (case, observer tile, element range) from a device counter, largest first.  A case
 * whose records fit the mixed bin ring (or, in a case of more steps than its slots, a
 * wide ring of 1024 or 2048 slots) runs the ring form on that ring, the others whole rows (the tests of
 * acum_set_ring, per case).  The tile shape -- observers per block, observers per warp,
 * elements per pipeline stage, work items per SM -- is set by acum_batch_set_tile /
 * acum_batch_set_tile2 or chosen by acum_batch_autotune (default 32 observers per block,
 * two per warp, 8 elements per stage; fewer observers per block where the longest rows
 * leave no room for 32, and one per warp where two would leave fewer than 12 warps). */
typedef struct acum_batch acum_batch;

int acum_batch_create(acum_batch** out, int device);
int acum_batch_destroy(acum_batch* b);
const char* acum_batch_last_error(const acum_batch* b);
/* Adds a case (same argument meaning as acum_set_deck with host rows) and preprocesses it
 * on the device at once; the rows are not kept, only the mixed-form records (2048 bytes
 * per element and window of 31 steps).  Fails with ACUM_ERR_NOMEM, adding nothing, when the
 * device has less free memory than the case needs plus 1 GiB.  *case_id = its index. */
int acum_batch_add(acum_batch* b, const acum_inputs* in, int nobs, const float* obs_file, int nsurf,
                   const int* nelem, const float* raw, int* case_id);
int acum_batch_count(const acum_batch* b, int* ncase);
/* Builds the work list for the current tile shape (done by acum_batch_run if needed). */
int acum_batch_prepare(acum_batch* b);
/* precision must be ACUM_MIXED.  mode 0: one persistent launch over all cases (plus
 * one zeroing of the sums and one finalize launch); 1: one launch per case (the
 * single-deck path, case after case on one stream); 2: mode 0 captured once into a CUDA
 * graph and replayed. */
int acum_batch_run(acum_batch* b, int precision, int mode);
/* pA [nTime_c][nObs_c] of one case after a run, host memory. */
int acum_batch_result(acum_batch* b, int case_id, double* pA);
/* Device time of the last run (CUDA events on the batch's stream around all of its
 * work) and the number of kernels it launched. */
int acum_batch_timing(const acum_batch* b, double* ms, long long* launches);
/* Device time of one case's tonal kernel in the last mode-1 run. */
int acum_batch_case_timing(const acum_batch* b, int case_id, double* ms);
/* One observer per warp: obs_per_block 1..16, elems_per_stage 2, 4 or 8, items_per_sm >= 1
 * (0 keeps a value; a kept obs_per_block above 16 becomes 16). */
int acum_batch_set_tile(acum_batch* b, int obs_per_block, int elems_per_stage, int items_per_sm);
/* As acum_batch_set_tile with obs_per_warp 1 or 2; two: obs_per_block 2..32 (even; 0 =
 * 32), elems_per_stage 2 or 4 (0 = 4). */
int acum_batch_set_tile2(acum_batch* b, int obs_per_block, int elems_per_stage, int items_per_sm, int obs_per_warp);
int acum_batch_get_tile(const acum_batch* b, int* obs_per_block, int* elems_per_stage, int* items_per_sm);
int acum_batch_get_obs_per_warp(const acum_batch* b, int* obs_per_warp);
/* Chooses the tile shape.  (1) For every observers-per-block in {8, 12, 16} x elements-per-
 * stage in {2, 4, 8} (one observer per warp) and {16, 24, 32} x {2, 4, 8} (two per warp)
 * whose shared memory fits, one persistent launch over a probe of
 * 128-element work items spread over all cases (about probe_per_sm items per SM; 0 = 8)
 * gives the kernel's throughput; the fastest shape is kept (where none fits the longest
 * rows, the default shape shrunk to fit them).  (2) Two probes of that shape
 * with 64- and 256-element items give its cost per work item and per evaluation, from
 * which the largest-first dynamic schedule of the real work list is simulated for
 * items_per_sm in {4, 8, 16, 32}; the shortest predicted makespan is kept and returned in
 * *best_ms. */
int acum_batch_autotune(acum_batch* b, int probe_per_sm, double* best_ms);

#ifdef __cplusplus
}
#endif
#endif /* ACUM_H */
