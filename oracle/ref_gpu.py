"""MEASUREMENT INFRASTRUCTURE ONLY (the reference's own GPU tonal kernel as a baseline).

Loads the reference's tonal kernel, `findPressureTimeHistory` (core.cu:18), compiled
unmodified for sm_103a by oracle/build_ref.sh into oracle/_ref/core_sm103a.cubin, and launches it through the CUDA driver API with the launch shape main.cu:194-236
computes (blocks of 8 steps x 4 observers x 8 elements, at most 512 blocks per axis), on
the reference's AoS arrays (variables.cu:54: Xham, Nham, Vham, PRham with the XPtr /
NPtr / VPtr / PRPtr offsets) of a synthetic deck.  The AoS fields are this library's
GPU preprocessing (acum_get_fields, the preprocess_imper restatement), rounded to float as
the reference stores them.  Times the kernel with CUDA events and prints one JSON line per
workload: the reference kernel's evaluations/s, this library's mixed and FP64 kernels on
the same deck and GPU, and the reference kernel's pA error against the FP64 form.

    python oracle/ref_gpu.py [--workload 0 1 2] [--observers N] [--budget-s S]

Workloads run in the order given; one whose reference-kernel time, predicted from the
rate of the previous one, exceeds the budget is skipped (the kernel runs to completion
once launched).  The launch shape needs nTime and each surface's element count to be
multiples of 8 and nObs a multiple of 4, so that the barriers inside its grid-stride
loops (core.cu:241, 249, 255) are reached by every thread of a block; decks that are not
are refused.

Never used by the product, the tests or bench.py.
"""
import argparse
import ctypes as C
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

ENTRY = b"_Z23findPressureTimeHistoryPfS_S_S_S_S_S_S_S_iPiS0_S0_S0_S0_iiffffS_f"


def driver():
    cu = C.CDLL("libcuda.so.1")
    for n in ("cuModuleLoad", "cuModuleGetFunction", "cuLaunchKernel", "cuModuleUnload", "cuGetErrorString"):
        getattr(cu, n).restype = C.c_int
    return cu


def check(cu, rc, what):
    if rc != 0:
        s = C.c_char_p()
        cu.cuGetErrorString(rc, C.byref(s))
        raise RuntimeError("%s: CUDA driver error %d %s" % (what, rc, s.value))


def load_kernel(cu):
    mod = C.c_void_p()
    name = "core_sm103a.cubin"
    path = os.path.join(HERE, "_ref", name)
    if not os.path.exists(path):
        raise RuntimeError("reference kernel not built (oracle/_ref/%s missing)" % name)
    check(cu, cu.cuModuleLoad(C.byref(mod), path.encode()), "cuModuleLoad")
    fn = C.c_void_p()
    check(cu, cu.cuModuleGetFunction(C.byref(fn), mod, ENTRY), "cuModuleGetFunction")
    return mod, fn, name


def launch_shape(nTime, nObs):
    """main.cu:194-233"""
    ntpb_x, ntpb_y, ntpb_z, nb_max = 8, 4, 8, 512
    cround = lambda v: int(math.floor(v + 0.5))  # C round(): halves away from zero
    nb_t = min(cround(float(nTime // ntpb_x) + 0.5), nb_max)
    ntpb_t = ntpb_x
    if nTime < ntpb_t:
        ntpb_t, nb_t = nTime, 1
    nb_ob = min(cround(float(nObs // ntpb_y) + 0.5), nb_max)
    ntpb_ob = ntpb_y
    if nObs < ntpb_ob:
        ntpb_ob, nb_ob = nObs, 1
    return (nb_t, nb_ob, nb_max), (ntpb_t, ntpb_ob, ntpb_z)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", type=int, nargs="+", default=[0, 1])
    ap.add_argument("--observers", type=int, default=0, help="observer sample (every k-th), 0 = all")
    ap.add_argument("--budget-s", type=float, default=60.0)
    args = ap.parse_args()
    rate = None
    for w in args.workload:
        rate = run(w, args.observers, args.budget_s, rate)


def run(workload, observers, budget_s, rate):
    import torch
    from acum3_periodic_gb300 import native, synth

    d = synth.config_deck(workload)
    if observers and observers < d.nObs:
        d = d.subset_observers(np.arange(0, d.nObs, d.nObs // observers)[:observers])
    T, O = d.nTime, d.nObs
    if T % 8 or O % 4 or any(n % 8 for n in d.elements):
        print(json.dumps({"workload": workload, "skipped": "nTime, nObs or an element count not a multiple of "
                                                            "the reference's block shape"}))
        return rate
    if rate is not None and d.tonal_evals() / rate > budget_s:
        print(json.dumps({"workload": workload, "skipped": "predicted %.0f s > budget %.0f s"
                          % (d.tonal_evals() / rate, budget_s)}))
        return rate
    der = d.derived()
    ctx = native.Context(0)
    ctx.set_deck(d, bb=False)
    fields = ctx.fields()  # [E][T][18] FP64
    ms_mixed, ms_f64 = [], []
    for prec, out in ((native.MIXED, ms_mixed), (native.PLAIN_FP64, ms_f64)):
        ctx.tonal(prec)
        for _ in range(2):
            ctx.tonal(prec)
            out.append(ctx.timing(0)[0])
    _, _, ref64 = ctx.tonal(native.PLAIN_FP64)

    torch.cuda.init()
    dev = torch.device("cuda", 0)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)
    i32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(dev)
    ne = d.elements
    off = np.cumsum([0] + ne[:-1])
    X, N, V, P = (f32(fields[:, :, a:b]) for a, b in ((0, 4), (4, 10), (10, 16), (16, 18)))
    XP, NP_, VP, PP = (i32(off * k * T) for k in (4, 6, 6, 2))
    E = i32(ne)
    robs = f32(d.observers())
    tobs = f32(np.arange(T, dtype=np.float32) * np.float32(der["dPsi"]))
    vinf = f32(der["vInf"])
    pT, pL, pA = (torch.zeros((T, O), dtype=torch.float32, device=dev) for _ in range(3))
    del fields

    cu = driver()
    mod, fn, which = load_kernel(cu)
    grid, block = launch_shape(T, O)
    vals = [C.c_void_p(t.data_ptr()) for t in (robs, tobs, pT, pL, pA, X, N, V, P)]
    vals += [C.c_int(d.nSurf)] + [C.c_void_p(t.data_ptr()) for t in (XP, NP_, VP, PP, E)]
    vals += [C.c_int(O), C.c_int(T), C.c_float(der["dPsi"]), C.c_float(der["dTau"]), C.c_float(der["a0"]),
             C.c_float(der["rhoRef"]), C.c_void_p(vinf.data_ptr()), C.c_float(der["oM"])]
    params = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    check(cu, cu.cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1], block[2], 0,
                                C.c_void_p(stream.cuda_stream), params, None), "cuLaunchKernel")
    e1.record(stream)
    e1.synchronize()
    ms_ref = e0.elapsed_time(e1)
    got = pA.double().cpu().numpy()
    cu.cuModuleUnload(mod)
    evals = d.tonal_evals()
    rms = np.sqrt(np.mean(ref64 ** 2, axis=0, keepdims=True))
    oas = lambda p: 10 * np.log10(np.mean(p ** 2, axis=0) / 4e-10)
    print(json.dumps({
        "workload": workload, "elements": d.E, "steps": T, "observers": O, "evals": evals,
        "reference_kernel": {"module": which, "grid": grid, "block": block, "ms": ms_ref,
                             "evals_per_s": evals / (ms_ref * 1e-3),
                             "pA_err_over_rms_vs_fp64_max": float(np.max(np.abs(got - ref64) / rms)),
                             "oaspl_err_db_vs_fp64_max": float(np.max(np.abs(oas(got) - oas(ref64))))},
        "mixed_kernel": {"ms": min(ms_mixed), "evals_per_s": evals / (min(ms_mixed) * 1e-3)},
        "fp64_kernel": {"ms": min(ms_f64), "evals_per_s": evals / (min(ms_f64) * 1e-3)},
        "mixed_over_reference": ms_ref / min(ms_mixed),
        "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}), flush=True)
    ctx.close()
    return evals / (ms_ref * 1e-3)


if __name__ == "__main__":
    main()
