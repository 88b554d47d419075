"""Benchmark of the tonal hot path on the large workload (workload 2: 4 blades x 8000
panels = 32000 elements, 1440 steps per revolution, 4096 observers; seeded synthetic
rotor, see acum3_periodic_gb300/synth.py).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

GB300 arm (default).  One step = one pass of the tonal path over the deck with the
surface rows already resident in HBM: GPU preprocessing (preprocess_imper) + the
mixed-precision tonal kernel (the ring kernel, and the wide-ring and whole-row kernels
launched behind it, which return at once on this deck) + the finalize transpose, i.e.
acum_tonal_device.
`value` is element*observer*step evaluations per second over K timed steps (inputs larger
than L2: 1.47 GB of surface rows and 3.08 GB of records per step).  `e2e` times the same
metric through acum_tonal_from_host_async: pinned host rows in, pA out, copies inside
(each step's copies overlap the previous step's solve).  The plain FP64 form is timed on
every 8th observer (512) of the same deck, and the mixed result is compared with it
there (OASPL dB and per-bin error).  `cpu_baseline` times the oracle port (the C
restatement of the reference path) on this host's cores on a bounded sample of the
same deck.  Further legs (each with its own switch): broadband (BPM) on the workload's
broadband deck, the adjoint on workload 3, the permeable preprocessing of an
8192-element data surface, and the batched persistent launch on workload 4.

Reference arm (--impl reference).  The reference's CPU implementation of the path: the
oracle port in oracle/acum_oracle.c (the reference's sources are not shipped with this
package, so its own build cannot be timed where the benchmark runs), all host threads, on bounded samples of
the same workload; rank 0 only under torchrun.

Multi-GPU: replicas (weak scaling) -- each rank solves the whole workload on its own
GPU; no collective on the data path; value = all ranks' evaluations / max rank time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "elem·obs·step evals/s: mixed vs FP64 at ≤0.05 dB OASPL; adjoint/fwd ratio"
ALG_FLOPS_PER_EVAL = 102  # FP ops per tonal evaluation (integrand + observer time + deposits)
# FP ops per broadband evaluation (section, observer, step, band) in the observer
# contraction: five component products and sums (packed over band pairs) and the tip term,
# 12, plus the observer geometry (~45 FP ops per section, step and observer) shared by the
# 42 bands, 1
BPM_FLOPS_PER_EVAL = 13
# DRAM bytes (read + write) of one workload-2 launch of the mixed kernel, measured with ncu
# (one pass: dram__bytes_read.sum + dram__bytes_write.sum: 11.66 GB + 8.20 GB); the FP64
# flushes of the FP32 bins and the reads they cause, the 3.08 GB of records being read
# about once
TONAL_TRAFFIC_BYTES = 19.86e9
WORKLOAD = "workload 2: 4-blade rotor, 32000 elements, 1440 steps/rev, 4096 observers, tonal mixed precision"


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return ws, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ws: int, evals_per_rank: float, steps: int, seconds_max: float) -> float:
    """Whole-job evaluations per second when every rank solves its own copy of the workload
    (replicas, weak scaling): all ranks' evaluations over the slowest rank's time."""
    return ws * evals_per_rank * steps / seconds_max


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms in the background."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.out = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in self.out:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


_SMS = {}


def nominal_fp32_peak(clocks, device: int = 0) -> float:
    """Nominal FP32 FMA rate in TFLOP/s: SMs x 128 FP32 lanes x 2 FLOP x the median SM
    clock sampled under load (the maximum clock when no sample was taken)."""
    if device not in _SMS:
        import torch
        _SMS[device] = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    return _SMS[device] * 128 * 2 * float(mhz) * 1e6 / 1e12


class StreamTimer:
    """CUDA events recorded on a context's own stream (the stream its runs are issued on),
    with the device synchronised on both sides of the timed region."""

    def __init__(self, ctx, device: int):
        import torch
        self.torch = torch
        self.ctx = ctx
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.ExternalStream(ctx.stream_ptr(), device=self.dev)
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)

    def start(self):
        self.ctx.sync()
        self.torch.cuda.synchronize(self.dev)
        self.e0.record(self.stream)

    def stop(self) -> float:
        """Seconds between start() and now on the context's stream."""
        self.e1.record(self.stream)
        self.e1.synchronize()
        self.ctx.sync()
        self.torch.cuda.synchronize(self.dev)
        return self.e0.elapsed_time(self.e1) * 1e-3


def cpu_baseline(deck, nobs_sample: int, nthreads: int):
    """The oracle port (C, FP64, reference algorithm) on the first `nobs_sample`
    observers of the deck, with `nthreads` host threads; returns evals/s and details."""
    from oracle import oracle as O
    sub = deck.subset_observers(np.arange(nobs_sample))
    inputs = O.TonalInputs(sub)
    t0 = time.perf_counter()
    fields = O.preprocess(sub, inputs)
    t1 = time.perf_counter()
    O.tonal(sub, nthreads=nthreads, fields=fields, inputs=inputs)
    t2 = time.perf_counter()
    evals = sub.E * sub.nTime * sub.nObs
    return evals / (t2 - t0), dict(evals=evals, seconds=t2 - t0, preprocess_s=t1 - t0)


def adjoint_leg(native, device):
    """Workload 3 (2 x 2400 elements, 360 steps, 256 observers): cost of the hand-written
    adjoint of J = sum_obs mean_bins pA^2 relative to the forward (kernel times by CUDA
    events on the launching stream), and the FP32 gradient's error against the FP64 one.
    The finite-difference check of the FP64 gradient lives in the GPU tests."""
    from acum3_periodic_gb300 import synth
    d = synth.config_deck(3)
    ctx = native.Context(device)
    ctx.set_deck(d, bb=False)
    res = {"workload": "workload 3: 2 x 2400 elements, 360 steps, 256 observers", "evals": d.tonal_evals()}
    for name, prec in (("fp64", native.PLAIN_FP64), ("mixed", native.MIXED)):
        ctx.tonal(prec)
        f = []
        a = []
        for _ in range(3):
            ctx.tonal(prec)
            f.append(ctx.timing(0)[0])
            J, gcp, gx, gn = ctx.adjoint(prec)
            a.append(ctx.timing(4)[0])
        fm, am = float(np.median(f)), float(np.median(a))
        res[name] = {"forward_kernel_ms": fm, "adjoint_kernel_ms": am, "adjoint_over_forward": am / fm}
        if name == "fp64":
            g64 = (J, gcp, gx, gn)
        else:
            res[name]["grad_rel_err_vs_fp64"] = float(max(np.linalg.norm(x - y) / np.linalg.norm(y)
                                                          for x, y in zip((gcp, gx, gn), g64[1:])))
    ctx.close()
    return res


PER_BYTES_PER_ELEMENT_STEP = 140  # float storage: 12 values read (x, y, z, ds, n, u, P, rho), 23 written
# FP64 instructions per element-step of per_prep_kernel with the filters on: 2 passes x 5
# series x 13-tap Gaussian (13 DADD + 9.625 DMUL: each product shared by two outputs of a
# run of 16) = 226.25, 14 central differences x (1 DADD + 1 DMUL + 4 DFMA + ...) ~ 84,
# scaling ~ 13 (SASS thread-instruction counters: DMUL 123.25, DADD 144, DFMA 56)
PER_FP64_INSTR_PER_ELEMENT_STEP = 323.25


def permeable_leg(native, device, steps=3, cpu=True, n_elem=8192, ntime=1440, fp64_peak_tflops=None):
    """Permeable-surface preprocessing (preprocess_per) of a data surface of `n_elem`
    elements (two surfaces) over `ntime` steps, filters on (the reference's default
    lowpass = 1), float storage as the reference's arrays: the device-resident call
    (acum_preprocess_per_device, CUDA events on its stream), the host call with host
    copies inside (acum_preprocess_per on pinned arrays), and the oracle port on a sample
    of elements (one host thread, as the reference's loop)."""
    import ctypes as C
    import torch
    from acum3_periodic_gb300 import synth
    ne = [n_elem // 2, n_elem - n_elem // 2]
    X, N, U, PR = synth.permeable_rows(7, ne, ntime)
    V = np.zeros_like(N)
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (X, N, V, U, PR)]
    # scalars as float, as the float entry point receives them
    args = tuple(float(np.float32(x)) for x in (1.0 / (ntime * 9.0), 340.0, 1.2, 0.08, 1.0)) + (1, 1)
    T = ntime
    off = np.concatenate([[0], np.cumsum(ne)[:-1]])
    ptrs = [np.ascontiguousarray(off * T * w, dtype=np.int32) for w in (4, 6, 6, 6, 4)]
    E = np.array(ne, np.int32)
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    lib = native.lib()
    dev = torch.device("cuda", device)
    pristine = [torch.from_numpy(a).to(dev) for a in arrs]
    work = [t.clone() for t in pristine]
    stream = torch.cuda.Stream(device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    element_steps = n_elem * T

    def device_call():
        rc = lib.acum_preprocess_per_device(*[C.c_void_p(t.data_ptr()) for t in work], 0, 2,
                                            *[vp(q) for q in ptrs], vp(E), T, *args, C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise native.AcumError(rc, lib.acum_last_global_error().decode())

    dms = []
    for i in range(3 + steps):
        for w, p in zip(work, pristine):
            w.copy_(p)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        device_call()
        e1.record(stream)
        e1.synchronize()
        if i >= 3:
            dms.append(e0.elapsed_time(e1))
    dev_ms = float(np.mean(dms))
    got = [t.cpu().numpy() for t in work]
    # host arrays in, host arrays out, through the reference-shaped entry point
    pinned = [native.PinnedBuffer(a.shape, np.float32) for a in arrs]
    hs = []
    for i in range(1 + steps):
        for pb, a in zip(pinned, arrs):
            pb.array[...] = a
        t0 = time.perf_counter()
        rc = lib.acum_preprocess_per(*[C.c_void_p(pb.ptr) for pb in pinned], 2, *[vp(q) for q in ptrs], vp(E), T,
                                     *args)
        hs.append(time.perf_counter() - t0)
        if rc != 0:
            raise native.AcumError(rc, lib.acum_last_global_error().decode())
    host_equal = all(np.array_equal(pb.array, g) for pb, g in zip(pinned, got))
    for pb in pinned:
        pb.close()
    host_s = float(np.mean(hs[1:]))
    nbytes = int(sum(a.nbytes for a in arrs))
    out = {"workload": "permeable data surface: %d elements (2 surfaces), %d steps, filters on, periodic "
                       "derivatives, float storage" % (n_elem, T),
           "element_steps": element_steps, "device_call_ms": dev_ms,
           "element_steps_per_s": element_steps / (dev_ms * 1e-3),
           "hbm_view": {"algorithmic_bytes": element_steps * PER_BYTES_PER_ELEMENT_STEP,
                        "achieved_gbs": element_steps * PER_BYTES_PER_ELEMENT_STEP / (dev_ms * 1e-3) / 1e9},
           "e2e": {"ms": host_s * 1e3, "element_steps_per_s": element_steps / host_s, "h2d_bytes": nbytes,
                   "d2h_bytes": nbytes, "api": "acum_preprocess_per (pinned host arrays in and out)"},
           "host_call_equals_device_call": bool(host_equal)}
    if fp64_peak_tflops:
        # the FP64 pipe bounds the kernel: its instruction rate (one instruction per FMA)
        instr = PER_FP64_INSTR_PER_ELEMENT_STEP * element_steps / (dev_ms * 1e-3)
        peak = fp64_peak_tflops * 1e12 / 2.0
        out["roofline"] = {"bound": "fp64", "achieved": instr, "peak": peak, "unit": "FP64 instructions/s",
                           "frac": instr / peak,
                           "fp64_instructions_per_element_step": PER_FP64_INSTR_PER_ELEMENT_STEP,
                           "peak_source": "measured FP64 FMA throughput of this GPU (acum_measure_peak), "
                                          "one instruction per FMA; the time is the whole device call"}
    if cpu:
        from oracle import oracle as O
        ns = min(2048, n_elem)
        f64 = lambda a: a[:ns].astype(np.float64)
        t0 = time.perf_counter()
        want = O.preprocess_per(f64(arrs[0]), f64(arrs[1]), f64(arrs[3]), f64(arrs[4]), *args)
        cpu_s = time.perf_counter() - t0
        out["bit_equal_to_oracle_sample"] = bool(all(
            np.array_equal(g[:ns], w.astype(np.float32)) for g, w in zip(got, want)))
        out["cpu_baseline"] = {"element_steps_per_s": ns * T / cpu_s, "cores": 1, "kind": "port",
                               "sample": "first %d of %d elements, all steps (oracle preprocess_per, FP64)" % (
                                   ns, n_elem)}
    return out


def profile_case(name, device=0):
    """One small run of one kernel family, for ncu captures of single launches:
    adjoint-fp64 / adjoint-mixed: the forward and the adjoint on workload 3;
    bpm: the broadband kernels on workload 1's broadband deck (4 x 50 sections, 720
    steps, 1024 observers); batch: four workload-4 cases shrunk to 30 x 2 x 12 panels per
    blade and 400 observers (376 MB of records) in one persistent launch (32 observers per
    block, two per warp, 8 elements per stage, 8 items per SM); tonal-small: the mixed kernel on
    workload 2 reduced to 25 x 2 x 10 panels per blade and 512 observers; tonal-full: the
    mixed kernel on workload 2 (for one-pass captures only); tonal-long: hovering rotors
    of long periods (workload 0's blades at 40 x 2 x 10 panels, 1024 observers; 2048 steps
    at tip Mach 0.8 and 0.6, 4096 steps at tip Mach 0.6 and 0.9) on the plan's kernel and on
    whole rows asked for, median of 5 runs each, with their largest difference in units
    of the observer RMS."""
    from acum3_periodic_gb300 import native, synth
    out = {"case": name}
    if name.startswith("adjoint"):
        ctx = native.Context(device)
        ctx.set_deck(synth.config_deck(3), bb=False)
        J, *_ = ctx.adjoint(native.PLAIN_FP64 if name == "adjoint-fp64" else native.MIXED)
        out.update(J=J, adjoint_ms=ctx.timing(4)[0])
    elif name == "bpm":
        ctx = native.Context(device)
        ctx.set_deck(synth.config_deck(1))
        ctx.bpm(0)
        out.update(bpm_ms=ctx.timing(3)[0], contraction_ms=ctx.timing(6)[0])
    elif name == "batch":
        b = native.Batch(device)
        for c in (3, 9, 14, 27):
            b.add(synth.batch_deck(c, shrink=dict(n_span=30, n_chord_side=12, nobs=400)))
        b.set_tile(32, 8, 8, 2)
        b.run(mode=0)
        out.update(batch_ms=b.timing()[0])
    elif name == "tonal-long":
        ctx = native.Context(device)
        out["decks"] = []
        for T, tip in ((2048, 0.8), (4096, 0.6), (2048, 0.6), (4096, 0.9)):
            d = synth.config_deck(0, replicate=37, scale=dict(n_span=40, n_chord_side=10, ntime=T, nobs=1024,
                                                               tip_mach=tip, minf=0.0))
            ctx.set_deck(d, bb=False)
            row = {"steps": T, "tip_mach": tip, "evals": d.tonal_evals()}
            res = {}
            for rows in (0, 1):
                ctx.set_tile(whole_rows=rows)
                ctx.tonal(native.MIXED)
                ts = []
                for _ in range(5):
                    _, _, res[rows] = ctx.tonal(native.MIXED)
                    ts.append(ctx.timing(0)[0])
                ms = float(np.median(ts))
                plan = ctx.last_plan()
                row["whole_rows" if rows else "plan"] = {"ms": ms, "evals_per_s": row["evals"] / ms * 1e3,
                                                         "ring_used": plan["ring_used"]}
            ctx.set_tile()
            rms = np.sqrt(np.mean(res[1] ** 2, axis=0, keepdims=True))
            row["max_diff_over_rms"] = float((np.abs(res[0] - res[1]) / rms).max())
            out["decks"].append(row)
    else:
        ctx = native.Context(device)
        scale = None if name == "tonal-full" else dict(n_span=25, n_chord_side=10, ntime=1440, nobs=512)
        ctx.set_deck(synth.config_deck(2, scale=scale), bb=False)
        ctx.tonal(native.MIXED)
        out.update(tonal_ms=ctx.timing(0)[0])
    print(json.dumps(out))


PROFILE_CASES = ("adjoint-fp64", "adjoint-mixed", "bpm", "batch", "tonal-small", "tonal-full", "tonal-long")


def batch_leg(native, device, steps=1, inflight=6):
    """Workload 4: 64 seeded rotor cases (2-6 blades, 500-20000 elements per blade, 180-1440
    steps, 64-2048 observers) resident on the GPU and solved in mixed precision (a) by one
    persistent launch replayed from a CUDA graph, tile shape from the autotuner, and (b) by
    one launch per case.  Decks are generated on host threads (a bounded number in flight)
    and added one by one; only their records stay on the device.  The same comparison on
    64 small cases (the same draws capped at 10 x 2 x 8 panels per blade, 360 steps and
    128 observers), where one case fills a few SMs only, is in `small_cases`."""
    from acum3_periodic_gb300 import synth
    res = _batch_compare(native, device, lambda c: synth.batch_deck(c), steps, inflight)
    res["workload"] = "workload 4: 64 rotor cases, one persistent launch (CUDA graph) vs one launch per case"
    small = dict(n_span=10, n_chord_side=8, ntime=360, nobs=128)
    sm = _batch_compare(native, device, lambda c: synth.batch_deck(c, shrink=small), max(steps, 3), inflight)
    sm["workload"] = ("64 small rotor cases (workload 4 draws capped at %d x 2 x %d panels per blade, %d steps, "
                      "%d observers)" % (small["n_span"], small["n_chord_side"], small["ntime"], small["nobs"]))
    sm["per_case"].pop("per_case", None)
    sm["per_case"].pop("per_case_columns", None)
    res["small_cases"] = sm
    return res


def _batch_compare(native, device, make_deck, steps, inflight):
    from concurrent.futures import ThreadPoolExecutor
    from acum3_periodic_gb300 import synth
    ncase = len(synth.batch_specs())
    b = native.Batch(device)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(inflight) as ex:
        futs = [ex.submit(make_deck, c) for c in range(min(inflight, ncase))]
        nxt = len(futs)
        for c in range(ncase):
            d = futs[c].result()
            futs[c] = None
            b.add(d)
            del d
            if nxt < ncase:
                futs.append(ex.submit(make_deck, nxt))
                nxt += 1
    gen_s = time.perf_counter() - t0
    evals = np.array([e for (_, _, e) in b.shapes], np.float64)
    total = float(evals.sum())
    t0 = time.perf_counter()
    est_ms = b.autotune()
    tune_s = time.perf_counter() - t0
    tile = b.tile()
    res = {"cases": ncase, "evals": total, "deck_generation_s": gen_s, "autotune_s": tune_s,
           "tile": {"obs_per_block": tile[0], "elems_per_stage": tile[1], "items_per_sm": tile[2],
                    "obs_per_warp": b.obs_per_warp()},
           "autotune_estimate_ms": est_ms}
    for name, mode in (("persistent_graph", 2), ("per_case", 1)):
        b.run(mode=mode)
        ms = []
        for _ in range(steps):
            b.run(mode=mode)
            ms.append(b.timing()[0])
        m = float(np.median(ms))
        res[name] = {"ms": m, "evals_per_s": total / (m * 1e-3), "gpu_launches": b.timing()[1],
                     "fp32_tflops": ALG_FLOPS_PER_EVAL * total / (m * 1e-3) / 1e12}
        if mode == 1:
            case_ms = np.array([b.case_ms(i) for i in range(ncase)])
            per = evals / (case_ms * 1e-3)
            res[name]["per_case_evals_per_s"] = {"min": float(per.min()), "median": float(np.median(per)),
                                                 "max": float(per.max())}
            res["per_case"]["per_case"] = [[int(b.shapes[i][0]), int(b.shapes[i][1]), float(evals[i]),
                                            float(case_ms[i])] for i in range(ncase)]
            res["per_case"]["per_case_columns"] = ["nTime", "nObs", "evals", "kernel_ms"]
            last = [b.result(i) for i in (0, ncase // 2, ncase - 1)]
    b.run(mode=2)
    rms = lambda p, r: float(np.max(np.abs(p - r) / np.sqrt(np.mean(r ** 2, axis=0, keepdims=True))))
    res["persistent_vs_per_case_bin_err_over_rms_max"] = max(
        rms(b.result(i), r) for i, r in zip((0, ncase // 2, ncase - 1), last))
    res["speedup_persistent_over_per_case"] = res["per_case"]["ms"] / res["persistent_graph"]["ms"]
    b.close()
    return res


def run_reference(args, deck, ws, rank, dist):
    if rank != 0:
        return
    nth = os.cpu_count() or 1
    nobs = max(nth, 16)
    vals = []
    for i in range(args.warmup + args.steps):
        v, info = cpu_baseline(deck, nobs, nth)
        if i >= args.warmup:
            vals.append(info["seconds"])
    sec = float(np.mean(vals))
    evals = deck.E * deck.nTime * nobs
    value = evals / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded rotor deck)",
        "config": {"workload": WORKLOAD, "elements": deck.E, "steps": deck.nTime, "observers": deck.nObs},
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": nth, "kind": "port",
                         "sample": "first %d of %d observers x all %d elements x %d steps per step (%d evals); "
                                   "oracle/acum_oracle.c, FP64, %d threads" % (nobs, deck.nObs, deck.E, deck.nTime,
                                                                               evals, nth)},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-every", type=int, default=8, help="time the FP64 form on every n-th observer")
    ap.add_argument("--cpu-obs", type=int, default=16, help="observers in the CPU-baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--small", action="store_true", help="a reduced deck (for profiling runs)")
    ap.add_argument("--no-bpm", action="store_true", help="skip the broadband leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg (workload 3)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched leg (workload 4)")
    ap.add_argument("--no-permeable", action="store_true", help="skip the permeable preprocessing leg")
    ap.add_argument("--batch-steps", type=int, default=1, help="timed runs per mode of the batched leg")
    ap.add_argument("--case", choices=sorted(PROFILE_CASES), default=None,
                    help="run one small case of one kernel family once and exit (for ncu captures)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if not args.small else args.warmup

    if args.case:
        profile_case(args.case)
        return
    ws, rank, local, dist = dist_init()
    from acum3_periodic_gb300 import synth
    scale = dict(n_span=25, n_chord_side=10, ntime=1440, nobs=512) if args.small else None
    deck = synth.config_deck(2, scale=scale)

    if args.impl == "reference":
        run_reference(args, deck, ws, rank, dist)
        return

    from acum3_periodic_gb300 import native
    ctx = native.Context(local)
    ctx.set_deck(deck, bb=False)
    evals = deck.tonal_evals()

    def step():
        ctx.mark_surfaces_changed()
        ctx.tonal_device(native.MIXED, 0, 0, 0)

    for _ in range(args.warmup):
        step()
    ctx.sync()
    sampler = ClockSampler(local)
    sampler.start()
    kern_ms, prep_ms, fin_ms, launches = [], [], [], 0
    timer = StreamTimer(ctx, local)
    barrier(dist)
    timer.start()
    for _ in range(args.steps):
        step()
        kern_ms.append(ctx.timing(0)[0])
        prep_ms.append(ctx.timing(1)[0])
        fin_ms.append(ctx.timing(2)[0])
        launches += ctx.timing(0)[1]
    elapsed = max_over_ranks(dist, timer.stop())
    barrier(dist)
    clocks = sampler.stop()
    value = replica_throughput(ws, evals, args.steps, elapsed)
    ms_per_step = elapsed / args.steps * 1e3

    # end to end through the C ABI from pinned host memory
    raw = deck.raw_surfaces()
    pin_raw = native.PinnedBuffer(raw.shape, np.float32)
    pin_raw.array[:] = raw
    pin_pA = native.PinnedBuffer((deck.nTime, deck.nObs), np.float64)
    ctx.tonal_from_host(native.MIXED, pin_raw.ptr, pin_pA.ptr)
    barrier(dist)
    # one synchronous call for the copy share of a call, then the timed steps pipelined
    # (each step's rows copied while the previous step solves; every copy in the region)
    ctx.tonal_from_host(native.MIXED, pin_raw.ptr, pin_pA.ptr)
    call, prep_, kern_, fin_ = (ctx.timing(w)[0] for w in (5, 1, 0, 2))
    timer.start()
    for _ in range(args.steps):
        ctx.tonal_from_host_async(native.MIXED, pin_raw.ptr, pin_pA.ptr)
    ctx.sync()
    e2e_elapsed = max_over_ranks(dist, timer.stop())
    barrier(dist)
    e2e_value = replica_throughput(ws, evals, args.steps, e2e_elapsed)
    mixed_pA = np.array(pin_pA.array)

    # plain FP64 on every n-th observer of the same deck, and the accuracy of the mixed form
    sel = np.arange(0, deck.nObs, args.fp64_every)
    sub = deck.subset_observers(sel)
    ctx64 = native.Context(local)
    ctx64.set_deck(sub, bb=False)
    _, _, pA64 = ctx64.tonal(native.PLAIN_FP64)
    timer64 = StreamTimer(ctx64, local)
    timer64.start()
    ctx64.mark_surfaces_changed()
    ctx64.tonal_device(native.PLAIN_FP64, 0, 0, 0)
    fp64_sec = timer64.stop()
    fp64_kern = ctx64.timing(0)[0] / 1e3
    fp64_value = sub.tonal_evals() / fp64_sec
    ref = pA64
    mix = mixed_pA[:, sel]
    oas = lambda p: 10 * np.log10(np.mean(p ** 2, axis=0) / 4e-10)
    oaspl_err = float(np.max(np.abs(oas(mix) - oas(ref))))
    rms = np.sqrt(np.mean(ref ** 2, axis=0, keepdims=True))
    bin_rms_err = float(np.max(np.abs(mix - ref) / rms))
    scale_ = np.maximum(np.abs(ref), 1e-6 * np.abs(ref).max(axis=0, keepdims=True))
    bin_rel_err = float(np.median(np.abs(mix - ref) / scale_))

    # roofline of the dominant kernel (the mixed tonal kernel), CUDA-event timed
    kms = float(np.mean(kern_ms))
    fp32_peak = native.measure_peak(local, 0)
    fp64_peak = native.measure_peak(local, 1)
    achieved = ALG_FLOPS_PER_EVAL * evals / (kms * 1e-3) / 1e12
    rec_bytes = deck.E * deck.nTime * 16 * 4

    out = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded rotor deck)",
        "config": {"workload": WORKLOAD, "elements": deck.E, "steps": deck.nTime, "observers": deck.nObs,
                   "precision": "mixed", "l2": "inputs larger than L2 (1.47 GB rows, 2.95 GB records per step)",
                   "parallelism": "replicas" if ws > 1 else "1 GPU"},
        "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": int(raw.nbytes),
                "api": "acum_tonal_from_host_async (pinned rows in, pA out; copies overlap the previous step)",
                "synchronous_call_ms": call, "synchronous_copies_ms": call - prep_ - kern_ - fin_,
                "d2h_bytes_per_step": int(deck.nTime * deck.nObs * 8)},
        "gpu_launches": int(launches),
        "kernels_ms_per_step": {"preprocess": float(np.mean(prep_ms)), "tonal_mixed": kms,
                                "finalize": float(np.mean(fin_ms))},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": TONAL_TRAFFIC_BYTES,
                     "peak_nominal": nominal_fp32_peak(clocks, local),
                     "frac_of_nominal": achieved / nominal_fp32_peak(clocks, local),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one full-size "
                                       "launch of this kernel (bytes per launch; algorithmic: %d)" % rec_bytes,
                     "peak_source": "measured FP32 FMA throughput of this GPU (acum_measure_peak); "
                                    "MEASURED_PEAKS.json holds no CUDA-core FP32 peak",
                     "algorithmic_flops_per_eval": ALG_FLOPS_PER_EVAL,
                     "hbm_view": {"record_bytes_per_launch": rec_bytes,
                                  "achieved_gbs": rec_bytes / (kms * 1e-3) / 1e9}},
        "fp64": {"evals_per_s": fp64_value, "kernel_evals_per_s": sub.tonal_evals() / fp64_kern,
                 "observers": int(len(sel)), "fp64_peak_tflops": fp64_peak,
                 "kernel_frac_of_fp64_peak": ALG_FLOPS_PER_EVAL * sub.tonal_evals() / fp64_kern / 1e12 / fp64_peak},
        "mixed_over_fp64": value / fp64_value,
        "accuracy_vs_fp64": {"oaspl_max_err_db": oaspl_err, "per_bin_err_over_rms_max": bin_rms_err,
                             "per_bin_rel_err_median": bin_rel_err, "observers_compared": int(len(sel))},
        "clocks": clocks,
    }
    # broadband (BPM) path on the same workload's broadband deck (4 x 50 sections)
    if deck.BB_noise == 1 and not args.no_bpm:
        ctx.set_bb(deck)
        ctx.bpm(0)
        bt = []
        for _ in range(max(1, args.steps // 2)):
            timer.start()
            spl, oas = ctx.bpm(0)
            bt.append(timer.stop())
        bpm_kernel_ms = ctx.timing(3)[0]
        obs_ms = ctx.timing(6)[0]
        nsec = sum(b.nsect for b in deck.bb)
        bpm_evals = nsec * deck.nObs * deck.nTime * 42
        bsel = np.arange(0, deck.nObs, max(1, deck.nObs // 8))[:8]
        # gpu_ms: CUDA-event time of the six broadband kernels of one call (positions,
        # per-(section, step) preparation, spectra, observer contraction, dB sums, OASPL)
        bpm = {"metric": "section·observer·band evals/s (per source step)", "sections": nsec,
               "evals": bpm_evals, "evals_per_s": bpm_evals / float(np.mean(bt)),
               "gpu_evals_per_s": bpm_evals / (bpm_kernel_ms * 1e-3), "gpu_ms": bpm_kernel_ms,
               "per_section_observer_band_per_s": bpm_evals / float(np.mean(bt)) / deck.nTime}
        # roofline of the contraction kernel (bb_obs_kernel): FP32-pipe bound; its special
        # functions (one square root, two reciprocal square roots and two quotients per
        # observer, section and step) are 0.12 per evaluation, a small share of the XU rate
        bpm_ach = BPM_FLOPS_PER_EVAL * bpm_evals / (obs_ms * 1e-3) / 1e12
        bpm["roofline"] = {"kernel": "bb_obs_kernel", "bound": "fp32", "kernel_ms": obs_ms,
                           "achieved": bpm_ach, "unit": "TFLOP/s", "algorithmic_flops_per_eval": BPM_FLOPS_PER_EVAL,
                           "peak": fp32_peak, "frac": bpm_ach / fp32_peak,
                           "peak_nominal": nominal_fp32_peak(clocks, local),
                           "frac_of_nominal": bpm_ach / nominal_fp32_peak(clocks, local),
                           "xu_ops_per_eval": 5.0 / 42.0}
        if not args.no_cpu:
            from oracle import oracle as O
            sub = deck.subset_observers(bsel)
            nth = os.cpu_count() or 1
            t0 = time.perf_counter()
            ospl, ooas = O.bpm(sub, aa_mode=0, nthreads=nth)
            cpu_s = time.perf_counter() - t0
            bpm["oaspl_max_err_db"] = float(np.max(np.abs(oas[bsel] - ooas)))
            bpm["band_total_max_err_db"] = float(np.max(np.abs(spl[bsel, :, 0] - ospl[:, :, 0])))
            bpm["cpu_baseline"] = {"evals_per_s": nsec * len(bsel) * deck.nTime * 42 / cpu_s, "cores": nth,
                                   "kind": "port", "sample": "%d observers x all sections, steps, bands" % len(bsel)}
        out["bpm"] = bpm
    if not args.no_adjoint:
        out["adjoint"] = adjoint_leg(native, local)
    if not args.no_permeable:
        out["permeable"] = permeable_leg(native, local, steps=max(1, args.steps // 2), cpu=not args.no_cpu,
                                         n_elem=2048 if args.small else 8192, fp64_peak_tflops=fp64_peak)
    if rank == 0 and not args.no_cpu:
        nth = os.cpu_count() or 1
        v, info = cpu_baseline(deck, args.cpu_obs, nth)
        out["cpu_baseline"] = {"value": v, "unit": "evals/s", "cores": nth, "kind": "port",
                               "sample": "first %d of %d observers x all elements x all steps (%d evals), "
                                         "oracle/acum_oracle.c FP64 incl. its preprocessing" % (
                                             args.cpu_obs, deck.nObs, info["evals"])}
    pin_raw.close()
    pin_pA.close()
    ctx.close()
    ctx64.close()
    if not args.no_batch:
        try:
            out["batch"] = batch_leg(native, local, args.batch_steps)
        except native.AcumError as e:  # e.g. not enough device memory for all cases
            out["batch"] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
