"""Benchmark of the RI-K exchange step on one GB300.

Workload (synthetic RI-K system, seeded): 40 atoms uniform in a 12 Angstrom
box, 24 basis and 84 auxiliary functions per atom (n_bf 960, n_aux 3360),
n_occ 200, block size 24, tau 1e-10.  One step is the reference's exchange
pipeline: the 3c->2c transform B = X * V^{-1/2} on the compressed
significant-pair integrals (3c_2c_transform.cpp:44-57) followed by the occ-RI-K
step K = sum_{P,i} (mu i|P)[(ij|P)+(ji|P)] (occ_ri_k_step.cpp:83-130).

Metric: effective TFLOP/s = dense-equivalent FLOPs of the step
(2*n_vec2*n_aux^2 + 2*(n_bf^2*n_occ*n_aux + 2*n_bf*n_occ^2*n_aux), the
counts the reference's drivers print) / step time; higher is better.

`value`: inputs resident in HBM, device-timed with CUDA events on the
library's stream.  `e2e`: the same step through the C ABI with host buffers
(pinned), host->device copies and the K read-back inside the timed region.
`--impl reference` times the reference's CPU algorithm (the C oracle port,
OpenMP over P partitions, dgemm through OpenBLAS) on the host cores, on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG = dict(n_atoms=40, nbf=24, naux=84, n_occ=200, box=12.0, bs=24, thresh=1e-10, seed=42)
METRIC = "RI-K step time & eff. TFLOP/s: mixed vs FP64 GPU form at rel err ≤1e-9"
WORKLOAD = ("RI-K exchange step (3c->2c transform + occ-RI-K), 40 atoms in 12 A box, n_bf 960, n_aux 3360, n_occ 200,"
            " bs 24, tau 1e-10")


def step_flops(n_bf, n_aux, n_occ, n_vec2):
    f3c = 2.0 * n_vec2 * n_aux * n_aux  # 3c_2c_transform.cpp:52
    focc = 2.0 * (n_bf * n_bf * n_occ * n_aux + 2.0 * n_bf * n_occ * n_occ * n_aux)  # occ_ri_k_step.cpp:75
    return f3c, focc


def flops_total(n_bf, n_aux, n_occ, n_vec2):
    return sum(step_flops(n_bf, n_aux, n_occ, n_vec2))


class Clocks:
    """nvidia-smi samples during the timed region"""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                   r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def make_system(n_atoms=None):
    """the benchmark system; a smaller one (same density of atoms per volume)
    when n_atoms is given, for profiler captures"""
    from strassen_gb300 import synth as S

    if not n_atoms or n_atoms == CFG["n_atoms"]:
        return S.RikSystem(seed=CFG["seed"], n_atoms=CFG["n_atoms"], nbf=CFG["nbf"], naux=CFG["naux"],
                           n_occ=CFG["n_occ"], box=CFG["box"])
    box = CFG["box"] * (n_atoms / CFG["n_atoms"]) ** (1.0 / 3.0)
    return S.RikSystem(seed=CFG["seed"], n_atoms=n_atoms, nbf=CFG["nbf"], naux=CFG["naux"], n_occ=5 * n_atoms, box=box)


def cpu_sample(sysm, Xr, Bp, V, C):
    """The reference CPU algorithm (oracle port, OpenMP over P partitions,
    dgemm through OpenBLAS) on a bounded sample: the 3c->2c transform of the
    integral rows Xr and the occ-RI-K step on the transformed columns Bp.
    Returns (dense-equivalent flops, seconds, threads)."""
    from oracle import oracle as O

    O.enable_fast_gemm(True)
    bs, thr = CFG["bs"], CFG["thresh"]
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    O.transform_3c2c(Xr, V, bs, thr)
    t1 = time.perf_counter()
    O.rik_occ_step(Bp, sysm.keys, C, sysm.n_bf, Bp.shape[1], sysm.n_occ, bs, thr, cores)
    t2 = time.perf_counter()
    O.enable_fast_gemm(False)
    n_rows, n_p = Xr.shape[0], Bp.shape[1]
    f3c = 2.0 * n_rows * sysm.n_aux * sysm.n_aux
    focc = 2.0 * (sysm.n_bf ** 2 * sysm.n_occ * n_p + 2.0 * sysm.n_bf * sysm.n_occ ** 2 * n_p)
    return f3c + focc, t2 - t0, cores


def occ_sample_input(sysm, V, n_p):
    """B[:, :n_p] = X V^{-1/2}[:, :n_p] for the occ-RI-K sample (setup, untimed;
    X generated in P chunks with the bit-identical torch generator)"""
    import torch

    out = np.zeros((sysm.n_vec2, n_p))
    for p0 in range(0, sysm.n_aux, 256):
        p1 = min(sysm.n_aux, p0 + 256)
        Xc = sysm.ints_3c_torch("cpu", p0, p1).numpy().T
        out += Xc @ V[p0:p1, :n_p]
    return np.asfortranarray(out)


def screen_report(api, X, V, C, keys, B, sysm, bs, thr, d3, docc, ctx):
    """Screening of the two forms, each through the whole pipeline on its own
    3c->2c output, product by product: surviving block triples of both forms,
    flips (a triple kept by one form and dropped by the other) with the
    smallest and largest margin |est - thr| / thr among them, the smallest
    margin of any live triple, and block-level mask differences of mui_P,
    ij_P and ijs_P.  The 3c->2c and the mui = U C screens use norms of their
    inputs (X, V^{-1/2}; U_P = the 3c->2c output, C)."""
    from strassen_gb300 import screen

    n_bf, n_aux, n_occ = sysm.n_bf, sysm.n_aux, sysm.n_occ
    out = {}
    tr = {}
    for tag, form, nd3, ndo in (("mixed", api.FORM_OZAKI, d3, docc), ("fp64", api.FORM_FP64, 0, 0)):
        _, n3 = api.transform_3c2c(X, V, bs, thr, form=form, n_digits=nd3, out=B, ctx=ctx, stats=True)
        _, st, tr[tag] = api.rik_occ_step(B, keys, C, n_bf, n_aux, n_occ, bs, thr, n_part=1, form=form, n_digits=ndo,
                                          ctx=ctx, trace=True)
        out[tag] = {"3c2c": n3, "mui": st[0], "ij": st[1], "K": st[2]}
    cmp = screen.compare(tr["fp64"], tr["mixed"])
    rep = {}
    for prod in ("3c2c", "mui", "ij", "K"):
        r = {"surviving_fp64": out["fp64"][prod], "surviving_mixed": out["mixed"][prod]}
        if prod in cmp:
            r.update(flips=cmp[prod]["flips"], flip_margin_min=cmp[prod]["flip_margin_min"],
                     flip_margin_max=cmp[prod]["flip_margin_max"], margin_min_all_triples=cmp[prod]["margin_min_all"])
        rep[prod] = r
    rep["blocks"] = cmp["blocks"]
    rep["what"] = ("whole pipeline, each form on its own 3c->2c output; ij and K triples recounted on the host from "
                   "both forms' per-P block norms (margin = |norm product - thr| / thr, thr = tau bs^3)")
    return rep


def cpu_sample_sizes(cores):
    """Bounded sample that keeps every host core busy: 3c->2c on 16 rows of
    the port's 512-element super-blocks per core (16 x 22 block rows of 24
    integral rows; the super-block loop is the port's parallel loop), and the
    occ-RI-K step on 16 aux functions per core (one P partition per core)."""
    return 16 * 22 * CFG["bs"], 16 * cores


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n_rows, n_p = cpu_sample_sizes(os.cpu_count() or 1)
    sysm = make_system()
    V = sysm.v_m12()
    C = sysm.c_occ()
    Xr = sysm.ints_3c_rows(0, n_rows)
    Bp = occ_sample_input(sysm, V, n_p)
    for _ in range(args.warmup):
        cpu_sample(sysm, Xr, Bp, V, C)
    times, flops, cores = [], 0.0, 1
    for _ in range(args.steps):
        f, t, cores = cpu_sample(sysm, Xr, Bp, V, C)
        times.append(t)
        flops = f
    t = statistics.median(times)
    v = flops / t / 1e12
    sample = (f"3c->2c on {n_rows} of {sysm.n_vec2} integral rows + occ-RI-K on {n_p} of {sysm.n_aux} aux functions "
              "(OpenMP over super-blocks and P partitions, dgemm via OpenBLAS), throughput extrapolated to the step")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": cores, "kind": "port", "sample": sample,
                             "extrapolated": True},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import torch

    from strassen_gb300 import api

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sysm = make_system(args.atoms)
    n_bf, n_aux, n_occ, n_vec2, bs, thr = sysm.n_bf, sysm.n_aux, sysm.n_occ, sysm.n_vec2, CFG["bs"], CFG["thresh"]
    form = api.FORM_OZAKI if args.form == "ozaki" else api.FORM_FP64
    d3, docc = args.digits_3c2c, args.digits_occ
    # inputs generated on the device (bit-identical to the numpy generator)
    Xt = sysm.ints_3c_torch(dev)  # n_aux x n_vec2 row-major == n_vec2 x n_aux column-major
    X = Xt.T
    V = torch.from_numpy(np.ascontiguousarray(sysm.v_m12().T)).to(dev).T
    C = torch.from_numpy(np.ascontiguousarray(sysm.c_occ().T)).to(dev).T
    keys = torch.from_numpy(sysm.keys.view(np.int64)).to(dev)
    B = torch.empty((n_aux, n_vec2), dtype=torch.float64, device=dev).T
    K = torch.empty((n_occ, n_bf), dtype=torch.float64, device=dev).T
    stream = torch.cuda.Stream(device=dev)
    ctx = api.Context(local, stream=stream.cuda_stream)

    def step(form_, stats=None):
        api.transform_3c2c(X, V, bs, thr, form=form_, n_digits=d3, out=B, ctx=ctx)
        if stats is not None:
            stats["3c2c"] = ctx.gemm_timing()
            stats["3c2c_stalls"] = ctx.gemm_stalls()
            ctx.set_timing(True)
        _, st = api.rik_occ_step(B, keys, C, n_bf, n_aux, n_occ, bs, thr, n_part=1, form=form_, n_digits=docc, out=K,
                                 ctx=ctx, stats=True)
        if stats is not None:
            stats["occ"] = ctx.gemm_timing()
            stats["occ_stalls"] = ctx.gemm_stalls()
            stats["nsig"] = st[:3]

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        l0 = ctx.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(local) as clk:
            with torch.cuda.stream(stream):
                e0.record(stream)
                for _ in range(steps):
                    fn()
                e1.record(stream)
            torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        ms = e0.elapsed_time(e1) / steps
        return ms, (ctx.launch_count() - l0) / steps, clk.summary()

    f3c, focc = step_flops(n_bf, n_aux, n_occ, n_vec2)
    ms, launches, clocks = timed(lambda: step(form), args.steps, args.warmup)
    Kc = K.cpu().numpy().copy()
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    # one instrumented step: CUDA events around every tensor-core launch
    gemm = {}
    if form == api.FORM_OZAKI:
        with torch.cuda.stream(stream):
            ctx.set_timing(True)
            step(form, gemm)
            ctx.set_timing(False)
    # e2e through the C ABI with pinned host buffers (timed before the FP64 comparison, whose
    # allocations would otherwise be released and mapped again inside the timed region)
    e2e_ms = h2d = d2h = e2e_parts = e2e_each = None
    if not args.no_e2e:
        Xh = torch.empty((n_aux, n_vec2), dtype=torch.float64, pin_memory=True)
        Xh.copy_(Xt)
        Vh = V.T.cpu().pin_memory()
        Ch = C.T.cpu().pin_memory()
        kh = keys.cpu().pin_memory()
        Kh = torch.empty((n_occ, n_bf), dtype=torch.float64, pin_memory=True)
        keys_d = torch.empty_like(keys)
        C_d = torch.empty((n_occ, n_bf), dtype=torch.float64, device=dev)

        parts = {"3c2c_host_X": [], "occ_host_K": []}

        def step_e2e():
            # both calls return once their results are in place (host clock per part)
            t0 = time.perf_counter()
            api.transform_3c2c(Xh.T.numpy(), Vh.T.numpy(), bs, thr, form=form, n_digits=d3, out=B, ctx=ctx)
            t1 = time.perf_counter()
            keys_d.copy_(kh, non_blocking=True)
            C_d.copy_(Ch, non_blocking=True)
            api.rik_occ_step(B, keys_d, C_d.T, n_bf, n_aux, n_occ, bs, thr, n_part=1, form=form, n_digits=docc,
                             out=Kh.T.numpy(), ctx=ctx)
            parts["3c2c_host_X"].append(1e3 * (t1 - t0))
            parts["occ_host_K"].append(1e3 * (time.perf_counter() - t1))

        # each step timed on its own (CUDA events on the context's stream), the
        # median reported: the host link is shared with the other GPUs' jobs,
        # and single steps of an otherwise steady run take 2-5x as long
        e2e_steps = max(5, args.steps)
        step_e2e()  # warm-up
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        e2e_each = []
        with torch.cuda.stream(stream):
            for _ in range(e2e_steps):
                a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                step_e2e()
                a1.record(stream)
                torch.cuda.synchronize(dev)
                e2e_each.append(a0.elapsed_time(a1))
        if world > 1:
            torch.distributed.barrier()
        e2e_ms = float(np.median(e2e_each))
        e2e_parts = {k: float(np.median(v[-e2e_steps:])) for k, v in parts.items()}
        print("e2e parts per step (ms):", json.dumps(parts), file=sys.stderr)
        h2d = (Xh.numel() + Vh.numel() + Ch.numel() + kh.numel()) * 8
        d2h = Kh.numel() * 8
    extra = {}
    if form != api.FORM_FP64 and not args.skip_fp64:
        ms64, _, _ = timed(lambda: step(api.FORM_FP64), 1, 0)
        K64 = K.cpu().numpy()
        extra = {"fp64_ms_per_step": ms64, "speedup_vs_fp64": ms64 / ms,
                 "rel_err_vs_fp64": float(np.linalg.norm(Kc - K64) / np.linalg.norm(K64)),
                 "rel_err_bound": 1e-9}
        if not args.skip_kmn:
            # adjacent contraction: symmetric K_mn = sum_P mui_P mui_P^T on the same B (FP64 3c->2c output)
            Kmn = torch.empty((n_bf, n_bf), dtype=torch.float64, device=dev)
            st = {}

            def kmn_step(form_):
                st[form_] = api.rik_kmn_step(B, keys, C, n_bf, n_aux, n_occ, bs, thr, n_part=1, form=form_,
                                             n_digits=docc, out=Kmn, ctx=ctx, stats=True)[1]

            kms_oz, _, _ = timed(lambda: kmn_step(api.FORM_OZAKI), 1, 1)
            Kmn_oz = Kmn.cpu().numpy().copy()
            kms_64, _, _ = timed(lambda: kmn_step(api.FORM_FP64), 1, 0)
            Kmn_64 = Kmn.cpu().numpy()
            mprod = bs ** 3 * st[api.FORM_FP64][5]  # block products x bs^3 multiply-adds (bound: edge blocks smaller)
            extra["kmn"] = {"what": "K_mn = sum_P mui_P mui_P^T (n_bf x n_bf, lower blocks + mirror), mui_P recomputed",
                            "mixed_ms": kms_oz, "fp64_ms": kms_64, "speedup_vs_fp64": kms_64 / kms_oz,
                            "rel_err_vs_fp64": float(np.linalg.norm(Kmn_oz - Kmn_64) / np.linalg.norm(Kmn_64)),
                            "block_products": st[api.FORM_FP64][5], "mixed_block_products": st[api.FORM_OZAKI][5],
                            "kmn_product_flops_bound": 2.0 * mprod}
    if form != api.FORM_FP64 and not args.skip_fp64 and not args.skip_screen:
        extra["screen"] = screen_report(api, X, V, C, keys, B, sysm, bs, thr, d3, docc, ctx)
    if args.no_e2e:
        print(json.dumps({"metric": METRIC, "value": flops_total(n_bf, n_aux, n_occ, n_vec2) / (ms * 1e-3) / 1e12,
                          "unit": "TFLOP/s", "ms_per_step": ms, "note": "profiling run (no e2e / baselines)",
                          "n_vec2": n_vec2, "gemm": gemm}))
        return
    flops = f3c + focc
    value = world * flops / (ms * 1e-3) / 1e12
    peaks = measured_peaks()
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if form == api.FORM_FP64 else f"bf16x{d3}/{docc}-ozaki+f64",
            "data": "synthetic (seeded RI-K system, generated on device)",
            "config": {"workload": WORKLOAD + f"; n_vec2 {n_vec2}", "form": args.form,
                       "digits": {"3c2c": d3, "occ": docc} if form == api.FORM_OZAKI else None,
                       "l2": "inputs larger than L2 (X is %.1f GB)" % (n_vec2 * n_aux * 8 / 1e9)},
            "e2e": {"value": world * flops / (e2e_ms * 1e-3) / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "parts_ms": e2e_parts,
                    "timing": "median of per-step CUDA-event times", "ms_each": e2e_each},
            "gpu_launches": int(round(launches)), "clocks": clocks,
            "flops_split": {"3c2c": f3c, "occ": focc}}
    line.update(extra)
    if gemm:
        l3, ms3, m3 = gemm["3c2c"]
        lo, mso, mo = gemm["occ"]
        tri = lambda nd: nd * (nd + 1) // 2  # digit products per block product
        alg = 2.0 * (m3 * tri(d3) + mo * tri(docc))  # bf16 multiply-adds x2
        kms = ms3 + mso
        achieved = alg / (kms * 1e-3) / 1e12
        peak = peaks.get("bf16_tflops_sustained") or 1700.0
        # DRAM bytes (read + write) of the largest launch, the 3c->2c k_ozgemm, per launch like
        # `achieved`: dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of the full
        # workload's 3c->2c launch (two counters, one pass)
        traffic = 16.45e9 + 5.33e9 if args.atoms in (0, CFG["n_atoms"]) and d3 == 5 else None
        line["roofline"] = {"kernel": "k_ozgemm (tcgen05 digit-slice GEMM)", "bound": "tensor", "achieved": achieved,
                            "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                            "traffic_launch": "3c->2c k_ozgemm launch (23 ms), dram__bytes_read.sum + write.sum (one-pass ncu capture)",
                            "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained" if peaks else "fallback",
                            "launches_per_step": l3 + lo, "kernel_ms_per_step": kms,
                            "fp64_equivalent_tflops": 2.0 * (m3 + mo) / (kms * 1e-3) / 1e12,
                            "kernel_share_of_step": kms / ms,
                            "algorithmic": "2 * sum over surviving block triples of m*n*k * digit products"}
    else:
        line["roofline"] = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        Vn = np.asfortranarray(V.T.cpu().numpy().T)
        Cn = np.asfortranarray(C.T.cpu().numpy().T)
        n_rows, n_p = cpu_sample_sizes(os.cpu_count() or 1)
        Bs = np.asfortranarray(B[:, :n_p].cpu().numpy())
        f, t, cores = cpu_sample(sysm, sysm.ints_3c_rows(0, n_rows), Bs, Vn, Cn)
        line["cpu_baseline"] = {"value": f / t / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                                "sample": f"3c->2c on {n_rows} of {n_vec2} integral rows + occ-RI-K on {n_p} of "
                                          f"{n_aux} aux functions (OpenMP over super-blocks and P partitions, dgemm "
                                          "via OpenBLAS), throughput extrapolated to the step",
                                "extrapolated": True}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_rik_large(args):
    """The large RI-K configuration: 125 atoms in a 20 A box (n_bf 3000,
    n_aux 10500, n_occ 500), uniform 24-wide blocks (the per-atom shells of
    sizes 8-32 are not modelled), tau swept over 1e-6 .. 1e-12.  Per tau: one
    timed mixed-form step on device-resident inputs (X is 45 GB), and errors
    against the FP64 form on a sixteenth of the work: the 3c->2c output on the
    first rows of X, and K of the whole pipeline over the first aux functions,
    with the screen comparison of that part (flips per product and their
    margins).  At tau 1e-10 the whole FP64 step is also timed once (about a
    minute) and the mixed step's whole K compared with its K.  A measurement
    case, not the bench line."""
    import torch

    from strassen_gb300 import api
    from strassen_gb300 import screen
    from strassen_gb300 import synth as S

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    t0 = time.time()
    sysm = S.RikSystem(seed=CFG["seed"], n_atoms=125, nbf=24, naux=84, n_occ=500, box=20.0)
    n_bf, n_aux, n_occ, n_vec2, bs = sysm.n_bf, sysm.n_aux, sysm.n_occ, sysm.n_vec2, CFG["bs"]
    Xt = sysm.ints_3c_torch(dev)  # n_aux x n_vec2 row-major == n_vec2 x n_aux column-major
    X = Xt.T
    V = torch.from_numpy(np.ascontiguousarray(sysm.v_m12().T)).to(dev).T
    Cn = sysm.c_occ()
    C = torch.from_numpy(np.ascontiguousarray(Cn.T)).to(dev).T
    keys = torch.from_numpy(sysm.keys.view(np.int64)).to(dev)
    B = torch.empty((n_aux, n_vec2), dtype=torch.float64, device=dev).T
    K = torch.empty((n_occ, n_bf), dtype=torch.float64, device=dev).T
    setup_s = time.time() - t0
    ctx = api.Context(0)
    f3c, focc = step_flops(n_bf, n_aux, n_occ, n_vec2)
    rows = n_vec2 // 16
    # whole aux blocks: a ragged last block of V[:, :p_sub] would have another
    # block norm than the same columns inside the full V, and so another screen
    p_sub = (n_aux // 16) // bs * bs
    Xs = np.asfortranarray(X[:rows].cpu().numpy())
    Vn = np.asfortranarray(V.cpu().numpy())
    res = []
    FULL_TAU = 1e-10  # the tau of the whole-step FP64 comparison
    K_mixed = None
    for thr in (1e-6, 1e-8, 1e-10, 1e-12):
        def step():
            api.transform_3c2c(X, V, bs, thr, form=api.FORM_OZAKI, n_digits=args.digits_3c2c, out=B, ctx=ctx)
            api.rik_occ_step(B, keys, C, n_bf, n_aux, n_occ, bs, thr, form=api.FORM_OZAKI, n_digits=args.digits_occ,
                             out=K, ctx=ctx)

        step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if thr == FULL_TAU:
            K_mixed = K.cpu().numpy().copy()
        # errors against the FP64 form: the 3c->2c output on the first sixteenth of
        # the rows, and K of the whole pipeline (both forms from the same X) over
        # the first sixteenth of the aux functions, which needs only those
        # columns of B: FP64 B[:, :p_sub] = X V[:, :p_sub]
        b_oz = api.transform_3c2c(Xs, Vn, bs, thr, form=api.FORM_OZAKI, n_digits=args.digits_3c2c, ctx=ctx)
        b_64 = api.transform_3c2c(Xs, Vn, bs, thr, ctx=ctx)
        # FP64 form of those columns: matmult on block-sparse copies at threshold 0
        # with the output pre-filled with zeros, as 3c_2c_transform.cpp:44-57 does
        Xb = api.BlockSparseMatrix.from_dense(X, bs, bs, 0.0, ctx=ctx)
        Vb = api.BlockSparseMatrix.from_dense(V[:, :p_sub], bs, bs, 0.0, ctx=ctx)
        Cb = api.BlockSparseMatrix(n_vec2, p_sub, bs, bs, 0.0, ctx=ctx)
        Cb.fill_with_values(0.0)
        api.matmult(Cb, Xb, 0, Vb, 0, thr, 1.0, 1.0)
        del Xb, Vb
        B64 = torch.empty((p_sub, n_vec2), dtype=torch.float64, device=dev).T
        Cb.to_matrix(out=B64)
        del Cb
        # with the screen trace: per-product flips between the two pipelines
        k_64, st64, tr64 = api.rik_occ_step(B64, keys, C, n_bf, p_sub, n_occ, bs, thr, ctx=ctx, trace=True,
                                            out=torch.empty((n_occ, n_bf), dtype=torch.float64, device=dev).T)
        k_64 = k_64.cpu().numpy()
        del B64
        k_oz, stoz, troz = api.rik_occ_step(B[:, :p_sub], keys, C, n_bf, p_sub, n_occ, bs, thr, form=api.FORM_OZAKI,
                                            n_digits=args.digits_occ, ctx=ctx, trace=True,
                                            out=torch.empty((n_occ, n_bf), dtype=torch.float64, device=dev).T)
        k_oz = k_oz.cpu().numpy()
        cmp = screen.compare(tr64, troz, chunk=32)
        rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
        res.append({"tau": thr, "ms_per_step": ms, "tflops_dense_equiv": (f3c + focc) / (ms * 1e-3) / 1e12,
                    "rel_err_3c2c_rows_1_16": rel(b_oz, b_64), "rel_err_K_aux_1_16": rel(k_oz, k_64),
                    "screen_aux_1_16": {"mui_surviving": [st64[0], stoz[0]],
                                        "ij": cmp["ij"], "K": cmp["K"], "blocks": cmp["blocks"]}})
        del b_oz, b_64
    full = None
    if not args.skip_fp64:
        # the plain GPU FP64 form, whole step once at one tau (about a minute),
        # and the error of the mixed step's whole K against it
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        api.transform_3c2c(X, V, bs, FULL_TAU, out=B, ctx=ctx)
        api.rik_occ_step(B, keys, C, n_bf, n_aux, n_occ, bs, FULL_TAU, out=K, ctx=ctx)
        e1.record()
        torch.cuda.synchronize()
        fp64_ms = e0.elapsed_time(e1)
        K64 = K.cpu().numpy()
        mixed_ms = next(r["ms_per_step"] for r in res if r["tau"] == FULL_TAU)
        full = {"tau": FULL_TAU, "fp64_ms_per_step": fp64_ms, "mixed_ms_per_step": mixed_ms,
                "speedup_vs_fp64": fp64_ms / mixed_ms,
                "rel_err_K_vs_fp64": float(np.linalg.norm(K_mixed - K64) / np.linalg.norm(K64))}
    print(json.dumps({"metric": "large RI-K step, mixed form, per tau", "unit": "ms", "full_step_fp64": full,
                      "config": {"workload": f"125 atoms in a 20 A box, n_bf {n_bf}, n_aux {n_aux}, n_occ {n_occ}, "
                                             f"n_vec2 {n_vec2}, bs {bs} (uniform)",
                                 "digits": {"3c2c": args.digits_3c2c, "occ": args.digits_occ},
                                 "X_GB": n_vec2 * n_aux * 8 / 1e9}, "setup_s": setup_s,
                      "flops_dense_equiv": f3c + focc, "results": res}))


def run_batched(args):
    """Batched screened GEMMs (the batched-launch configuration): `--count`
    independent products C_i = A_i B_i, sizes uniform in [256, 4096] (rounded
    to the block size), block sizes from {16, 32, 48, 64}, block densities
    uniform in [0.05, 0.6], tau 1e-10; seeded inputs generated on the device.
    Mixed form: one persistent tensor-core launch over every block-size group
    (slots per tile autotuned per group), also replayed as a CUDA graph plan;
    FP64 form for reference.
    Metric: useful (FP64-equivalent) TFLOP/s of the surviving block products."""
    import torch

    from strassen_gb300 import api
    from strassen_gb300 import synth as S

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = api.Context(0)
    rng = np.random.default_rng(3)
    thr = 1e-10

    def mat(seed, stream, n, m, bs, dens):
        nbI, nbJ = -(-n // bs), -(-m // bs)
        keep = (S.uniform(S.stream_key(seed, stream + 1), np.arange(nbI * nbJ, dtype=np.uint64)).reshape(nbJ, nbI).T
                < dens)
        kt = torch.from_numpy(keep.astype(np.float64)).to(dev)
        idx = torch.arange(n * m, dtype=torch.int64, device=dev).reshape(m, n)  # [c, r] = r + c n
        g = S.gauss_torch(S.stream_key(seed, stream), idx)
        env = kt[torch.arange(n, device=dev) // bs][:, torch.arange(m, device=dev) // bs]  # n x m
        return (g * env.T).contiguous()  # (m, n) row-major = n x m column-major

    As, Bs, Cs, C64, bss, useful = [], [], [], [], [], 0.0
    for i in range(args.count):
        bs = int(rng.choice([16, 32, 48, 64]))
        m, k, n = (max(bs, int(rng.integers(256, 4097)) // bs * bs) for _ in range(3))
        da, db = float(rng.uniform(0.05, 0.6)), float(rng.uniform(0.05, 0.6))
        a = mat(1000 + i, 1, m, k, bs, da)
        b = mat(1000 + i, 2, k, n, bs, db)
        # input screen 1e-12: the all-zero blocks of the pattern are not stored
        As.append(api.BlockSparseMatrix(m, k, bs, bs, 1e-12, ctx=ctx, dense=a.T))
        Bs.append(api.BlockSparseMatrix(k, n, bs, bs, 1e-12, ctx=ctx, dense=b.T))
        Cs.append(api.BlockSparseMatrix(m, n, bs, bs, 0.0, ctx=ctx))
        C64.append(api.BlockSparseMatrix(m, n, bs, bs, 0.0, ctx=ctx))
        bss.append(bs)
        del a, b
    torch.cuda.synchronize()

    def timed(fn, reps):
        fn()  # warm-up (the first mixed-form call also tunes)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    nsig = api.matmult_batched(Cs, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI)
    t_mx = timed(lambda: api.matmult_batched(Cs, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI), args.steps)
    plan = api.BatchPlan(Cs, As, Bs, thr)
    t_plan = timed(plan.run, args.steps)
    t_64 = timed(lambda: api.matmult_batched(C64, As, Bs, thr, 1.0, 0.0, form=api.FORM_FP64), 1)
    # useful flops: the unpadded multiply-adds of the surviving block triples
    ctx.set_timing(True)
    api.matmult_batched(Cs, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI)
    gemm_launches, gemm_ms, macs = ctx.gemm_timing()
    ctx.set_timing(False)
    useful = 2.0 * macs
    errs = []
    for c, r in zip(Cs[:32], C64[:32]):
        x, y = c.to_matrix(), r.to_matrix()
        errs.append(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))
    line = {"metric": "batched screened GEMM throughput (useful FP64-equivalent TFLOP/s)",
            "value": useful / t_mx / 1e12, "unit": "TFLOP/s", "higher_is_better": True,
            "config": {"workload": f"{args.count} independent block-sparse GEMMs, sizes U[256,4096], block sizes "
                                   "{16,32,48,64}, block densities U[0.05,0.6], tau 1e-10 (seeded, generated on device)",
                       "surviving_block_triples": nsig, "useful_flops": useful},
            "mixed_ms": t_mx * 1e3, "plan_replay_ms": t_plan * 1e3, "plan_tflops": useful / t_plan / 1e12,
            "fp64_ms": t_64 * 1e3, "fp64_tflops": useful / t_64 / 1e12, "speedup_vs_fp64": t_64 / t_mx,
            "tensor_gemm_ms": gemm_ms, "tensor_gemm_launches": gemm_launches,
            "max_rel_err_first32": float(max(errs)),
            "autotune": {str(k): v for k, v in ctx.autotune_entries().items()}, "dtype": "bf16 digits (auto 4-5) + f64"}
    print(json.dumps(line))


STRASSEN_SHAPES = {
    # the Strassen benchmark's shape: n 2048, block 64, exp(-|I-J|/6), tau 1e-10, one Winograd level
    "n2048": dict(n=2048, bs=64, L=6.0, core=0, seed=1, thresh=1e-10, depths=(0, 1)),
    # the large shape: n 16384, block 64, dense core of the first 4096 rows and columns, exp(-|I-J|/10)
    # tails, tau 1e-9, Strassen depth 0..3
    "n16384": dict(n=16384, bs=64, L=10.0, core=4096, seed=4, thresh=1e-9, depths=(0, 1, 2, 3)),
    # a quarter of it (inputs still larger than L2), for profiler captures of the FP64 kernels
    "n8192": dict(n=8192, bs=64, L=10.0, core=2048, seed=4, thresh=1e-9, depths=(0, 1)),
}


def run_strassen(args):
    """Screened block GEMM and the hybrid Strassen-Winograd / sparse
    recursion (blocksparsematrix.hpp:293-414, strassen.hpp:687-753) at the
    Strassen benchmark's shapes.  Inputs are generated on the device (seeded,
    bit-identical to the host generator) and stored at threshold 0 as
    main.cpp stores them.  Per shape: the FP64 screened matmult, then
    matmult_strassen_sparse at each Strassen depth (min_size_for_strassen =
    n / 2^depth) in the FP64 and the mixed form (bf16 digits on the tensor
    cores; 4 digits at block 64), each timed after one warm-up call, with
    the relative error against the FP64 screened product.  TFLOP/s are
    dense-equivalent (2 n^3, as main.cpp:50 prints) and surviving-pair
    (2 bs^3 per surviving block triple).  A measurement case, not the bench
    line."""
    import torch

    from strassen_gb300 import api
    from strassen_gb300 import synth as S

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = api.Context(0)
    shapes = [args.shape] if args.shape else ["n2048", "n16384"]
    forms = ((api.FORM_FP64, "fp64"),) if args.fp64_only else ((api.FORM_FP64, "fp64"), (api.FORM_OZAKI, "mixed"))

    def timed(fn, reps=1):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps, r

    results = []
    for name in shapes:
        c = STRASSEN_SHAPES[name]
        n, bs, thr = c["n"], c["bs"], c["thresh"]
        a = S.decay_matrix_torch(c["seed"], 1, n, n, bs, c["L"], core=c["core"], device=dev)
        b = S.decay_matrix_torch(c["seed"], 2, n, n, bs, c["L"], core=c["core"], device=dev)
        A = api.BlockSparseMatrix.from_dense(a.T, bs, bs, 0.0, ctx=ctx)
        B = api.BlockSparseMatrix.from_dense(b.T, bs, bs, 0.0, ctx=ctx)
        del a, b
        dense_flops = 2.0 * n ** 3
        C64 = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
        t_mm, nsig = timed(lambda: api.matmult(C64, A, 0, B, 0, thr, 1.0, 0.0))
        surv_flops = 2.0 * nsig * bs ** 3
        R = C64.to_matrix()
        rn = np.linalg.norm(R)
        row = {"shape": name, "n": n, "bs": bs, "thresh": thr, "L": c["L"], "core": c["core"],
               "surviving_block_triples": nsig, "surviving_fraction": nsig / (n // bs) ** 3,
               "fp64_matmult_s": t_mm, "fp64_matmult_tflops_dense_equiv": dense_flops / t_mm / 1e12,
               "fp64_matmult_tflops_surviving": surv_flops / t_mm / 1e12, "strassen": []}
        if not args.fp64_only:
            Cz = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
            t_mz, _ = timed(lambda: api.matmult(Cz, A, 0, B, 0, thr, 1.0, 0.0, form=api.FORM_OZAKI, n_digits=0))
            row["mixed_matmult_s"] = t_mz
            row["mixed_matmult_rel_err"] = float(np.linalg.norm(Cz.to_matrix() - R) / rn)
            del Cz
        for d in c["depths"]:
            ms = n >> d
            ent = {"depth": d, "min_size_for_strassen": ms}
            # the reference's decision tree (cost model), then Strassen forced at
            # the root (the scheduler's ROOT policy) with the same depth below it
            for policy, ptag in ((api.SCHED_COST, ""), (api.SCHED_ROOT, "root_")):
                if policy == api.SCHED_ROOT and d == 0:
                    continue
                for form, tag in forms:
                    CS = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
                    nodes = [0]

                    def go():
                        CS.fill_with_values(0.0)
                        nodes[0] = api.matmult_strassen_sparse_sched(CS, A, B, thr, ms, policy, None, form, 0)

                    t, _ = timed(go)
                    key = ptag + tag
                    ent[key + "_s"] = t
                    ent[key + "_strassen_nodes"] = nodes[0]
                    ent[key + "_tflops_dense_equiv"] = dense_flops / t / 1e12
                    ent[key + "_rel_err_vs_fp64_matmult"] = float(np.linalg.norm(CS.to_matrix() - R) / rn)
                    del CS
            row["strassen"].append(ent)
        if name == "n2048" and not args.no_cpu_baseline:
            # the reference's CPU path (oracle port, dgemm through OpenBLAS) on the host cores
            from oracle import oracle as O

            ah = S.decay_matrix(c["seed"], 1, n, n, bs, c["L"], core=c["core"])
            bh = S.decay_matrix(c["seed"], 2, n, n, bs, c["L"], core=c["core"])
            oA, oB = O.OBsm(n, n, bs, bs, 0.0, ah), O.OBsm(n, n, bs, bs, 0.0, bh)
            O.enable_fast_gemm(True)
            oC = O.OBsm(n, n, bs, bs, 0.0)
            t0 = time.perf_counter()
            O.matmult(oC, oA, 0, oB, 0, thr)
            t_cpu = time.perf_counter() - t0
            O.enable_fast_gemm(False)
            row["cpu_baseline"] = {"kind": "port", "cores": os.cpu_count(), "matmult_s": t_cpu,
                                   "tflops_dense_equiv": dense_flops / t_cpu / 1e12,
                                   "what": "oracle port of the screened matmult, OpenMP over super-blocks, "
                                           "dgemm through OpenBLAS"}
        del A, B, C64
        torch.cuda.empty_cache()
        results.append(row)
    print(json.dumps({"metric": "screened block GEMM and hybrid Strassen-Winograd recursion, FP64 and mixed form",
                      "unit": "s", "data": "synthetic (seeded, generated on device)", "results": results}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="ozaki", choices=["fp64", "ozaki"])
    ap.add_argument("--digits-3c2c", type=int, default=5)
    ap.add_argument("--digits-occ", type=int, default=5)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-kmn", action="store_true", help="leave out the symmetric K_mn measurement")
    ap.add_argument("--skip-screen", action="store_true", help="leave out the per-product screening comparison")
    ap.add_argument("--no-e2e", action="store_true", help="profiling runs: timed device step only")
    ap.add_argument("--atoms", type=int, default=0, help="smaller system for profiler captures")
    ap.add_argument("--workload", default="rik", choices=["rik", "batched", "rik-large", "strassen"],
                    help="rik: the RI-K step (default); batched: the batched-GEMM configuration; strassen: the "
                         "screened GEMM and Strassen shapes")
    ap.add_argument("--shape", default="", choices=["", "n2048", "n16384", "n8192"],
                    help="strassen workload: one shape (default: n2048 and n16384)")
    ap.add_argument("--fp64-only", action="store_true", help="strassen workload: the FP64 form only")
    ap.add_argument("--count", type=int, default=512, help="products of the batched workload")
    args = ap.parse_args()
    if args.workload == "batched":
        run_batched(args)
        return
    if args.workload == "rik-large":
        run_rik_large(args)
        return
    if args.workload == "strassen":
        run_strassen(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
