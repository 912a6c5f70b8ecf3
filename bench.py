"""Benchmark: k-point H/S build + eigensolves per second on one GB300.

Workload (the configuration the metric is quoted on): fcc128, a 128-atom fcc
supercell with seeded 0.1 bohr displacements, spd basis (N = 1152), 3x3x3
Monkhorst-Pack mesh (27 k), mode 4.  One step = one full per-structure k loop
(the reference's bande call plus the search2 before it): neighbour list, SK
tables, H(k) and S(k), generalized eigensolve with vectors, dH/dV and dS/dV,
Hellmann-Feynman shifts, Fermi level, E(T) and P(T) for all 27 k.  k-point
solves/s = 27 / step time.

  value    device-resident: inputs staged in HBM before the timed region
           (nrltb_stage), K steps of nrltb_run timed with CUDA events on the
           library's stream.
  e2e      the same step through the reference-facing call nrltb_bande with
           host buffers (input upload and result download inside the region).
  fp64     the same step in the FP64 form (plain FP64 eigensolve), timed
           right after the mixed form in the same process; mixed_over_fp64 is
           the ratio, and fp64.mixed_vs_fp64 the mixed form's error against it
           over every k point (eigenvalues, E_F, E per atom, P in kbar).
  --impl reference
           the reference algorithm on the host cores: the C restatement in
           oracle/ (the Fortran reference cannot be compiled here), one k per
           thread on every host core this process may run on (its affinity
           mask), single-threaded LAPACK zhpgv per k.

The step's working set (H, S, dH, dS and the solver workspace for 27 k) is
several GB, far larger than L2, so no L2 flush is needed between steps.

--config batch256 times the structure batch instead: 256 seeded structures of
4-64 atoms (spd and sp3, N = 16-576) on 2^3-5^3 meshes, 14 525 k-point solves
per step, all through one nrltb_bande_batch call (host buffers).

--row selects the form of the same step for the rows beyond the path (the
default line is --row path): gillan (mode 2: entropy, E(0), P(0)), spin (a
two-set spin-polarized version of the parameters, two spin channels per k),
noncollinear (the two-set parameters with canted spin directions: one
2N x 2N problem per k), charges (mode 6: Lowdin orbital charges of every
state, downloaded in e2e).  Solves are counted per k and spin channel.
"""
import os

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")    # one LAPACK thread per k (before numpy)

import argparse
import json
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "tight-binding_gb300"))

METRIC = "k-point H/S build+eigensolves/s at N=1152, mixed vs FP64 on GB300 at 1e-9 Ry"
UNIT = "k-point solves/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(name):
    from nrltb import synth
    st, par, km, o = synth.CONFIGS[name]()
    return st, par, km, o


def workload_desc(name, st, par, km, row="path"):
    base = (f"{name}: {st.natoms}-atom supercell, N={par.nv(st)}, {km.nk} k, mode 4 "
            f"(H/S/dH/dS build, eigensolve with vectors, Hellmann-Feynman, E_F, E, P)")
    extra = {"path": "",
             "gillan": "; row gillan: mode 2 (also entropy, E(0), P(0))",
             "spin": "; row spin: two-set spin-polarized parameters, 2 channels per k",
             "noncollinear": "; row noncollinear: two-set parameters, canted spins, 2N x 2N per k",
             "charges": "; row charges: mode 6 (no pressure), Lowdin charges of every state"}[row]
    return base + extra


ROWS = ("path", "gillan", "spin", "noncollinear", "charges")


def row_setup(row, st, par):
    """(structure, parameters, mode, option flags, solves per k) of a row."""
    from dataclasses import replace
    import numpy as np
    from nrltb import synth
    if row == "path":
        return st, par, 4, 0, 1
    if row == "gillan":
        return st, par, 2, 0, 1
    mag = synth.magnetic_from(par)
    if row == "spin":
        return st, mag, 4, 0, 2
    if row == "noncollinear":
        # alternate the spin directions of the atoms over four canted orientations
        dirs = np.array([[0, 0, 1], [1, 0, 0], [0, 0.6, 0.8], [-0.6, 0, -0.8]], float)
        sp = dirs[np.arange(st.natoms) % 4]
        return replace(st, spinat=sp), mag, 4, 0, 1
    if row == "charges":
        return st, par, 6, 0, 1
    raise ValueError(row)


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        import statistics
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(rows), "reasons": reasons}


def cpu_sample(st, par, km, mode, nthreads, nk_sample, flags=0):
    """Oracle (reference algorithm) on the first nk_sample k points, all
    threads: (seconds, the oracle's result for those k points)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from nrltb import KMesh, Opts
    sub = KMesh(km.k[:nk_sample], km.w[:nk_sample] / km.w[:nk_sample].sum())
    opts = Opts(mode=mode, tkb=0.005, eigcut=1e3, flags=flags)
    t0 = time.perf_counter()
    r = oracle.bande(st, par, sub, opts, nthreads=nthreads)
    return time.perf_counter() - t0, r


def host_cores():
    """The host cores this process may run on (its affinity mask), which is
    what the container exposes; os.cpu_count() if the mask is unavailable."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    st0, par0, km, o = workload(args.config)
    st, par, mode, flags, per_k = row_setup(args.row, st0, par0)
    ncores = host_cores()
    nks = min(km.nk, ncores)
    times = []
    for i in range(args.warmup + args.steps):
        t, _ = cpu_sample(st, par, km, mode, ncores, nks, flags)
        if i >= args.warmup:
            times.append(t)
    mean = sum(times) / len(times)
    value = per_k * nks / mean
    sample = (f"{nks} of the {km.nk} k points per step (one per host thread), mode {mode}: setham + "
              f"zhpgv with vectors + sethamv + perturb, then Fermi/E/P")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded structure and parameters)",
            "config": {"workload": workload_desc(args.config, st0, par0, km, args.row), "host_cores": ncores,
                       "host_cores_note": "the cores this process may run on (its affinity mask)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


KCLASSES = [  # (class id, name, bound, unit of work, kernel name prefix in ncu)
    (0, "zgemm_umma_kernel / zgemm_tc_kernel: FP32 complex GEMM on the tensor cores (3xTF32; tcgen05 with "
        "tensor-memory accumulators for op(A) = A, mma.sync for op(A) = A^H)", "tensor", "flop", "zgemm_umma"),
    (1, "zgemm_kernel: complex GEMM on the FMA pipe (FP64 form; FP32 shapes below the tensor-core thresholds)",
     "fma", "flop", "zgemm_kernel"),
    (2, "k_oz_gemm: bf16 digit products on tcgen05 (refinement H X, S X to FP64 accuracy; Hellmann-Feynman "
        "dH Z, dS Z from 3-digit dH, dS)", "tensor", "flop", "k_oz_gemm"),
    (3, "k_tri_panel: tridiagonalisation panel (cluster per matrix, Hermitian mat-vec)", "hbm", "byte",
     "k_tri_panel"),
]


def kernel_stats(lib, ctx, steps):
    """Per-class totals of the timed region: ms per step, launches per step, work per step."""
    import ctypes as C
    out = []
    for cls, name, bound, unit, ncu_name in KCLASSES:
        ms, work, n = C.c_double(), C.c_double(), C.c_int()
        lib.nrltb_bench_kernel_stats(ctx.h, cls, C.byref(ms), C.byref(work), C.byref(n))
        if n.value == 0:
            continue
        rate = work.value / (ms.value * 1e-3)
        out.append({"class": cls, "kernel": name, "ncu_name": ncu_name, "bound": bound,
                    "ms_per_step": ms.value / steps,
                    "launches_per_step": n.value / steps,
                    ("tflops" if unit == "flop" else "gbs"): rate / (1e12 if unit == "flop" else 1e9),
                    "work_unit": unit})
    return out


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def pipe_peaks(lib, ctx):
    """Live microbenchmarks of the pipes MEASURED_PEAKS.json does not cover."""
    import ctypes as C
    pipe = {}
    for kind, name in ((0, "fp64_fma_tflops"), (1, "fp32_fma_tflops"), (2, "mma_sync_bf16_tflops"),
                       (3, "mma_sync_tf32_tflops"), (4, "l2_read_gbs")):
        t = C.c_double()
        if lib.nrltb_bench_peak(ctx.h, kind, C.byref(t)) == 0:
            pipe[name] = t.value
    return pipe


def profile_traffic(kernel_prefix):
    """DRAM bytes per launch of a kernel from a committed ncu summary: the
    summaries in profiles/ carry a line 'traffic_per_launch <kernel> <bytes>
    <what one launch processed>' taken from the capture they describe."""
    pdir = os.path.join(REPO, "profiles")
    try:
        names = sorted(os.listdir(pdir))
    except OSError:
        return None
    for f in names:
        if not f.endswith(".md"):
            continue
        with open(os.path.join(pdir, f)) as fh:
            for line in fh:
                parts = line.strip().strip("`").split(None, 3)
                if len(parts) >= 3 and parts[0] == "traffic_per_launch" and parts[1].startswith(kernel_prefix):
                    return {"bytes": float(parts[2]), "per": parts[3] if len(parts) > 3 else "",
                            "source": "profiles/" + f}
    return None


def roofline_of(kernels, prec, pipe):
    """Roofline entry of the class with the most time in the timed region."""
    if not kernels:
        return None
    dom = max(kernels, key=lambda k: k["ms_per_step"])
    peaks = measured_peaks()
    r = {"kernel": dom["kernel"], "ms_per_step": dom["ms_per_step"], "launches_per_step": dom["launches_per_step"],
         "traffic": None, "measured_live": "CUDA events around each launch of the class on the library stream, "
                                           "summed over K instrumented steps run right after the timed ones"}
    if dom["bound"] == "hbm":
        peak = peaks.get("hbm_gbs", 6800.0)
        r.update({"bound": "hbm", "achieved": dom["gbs"], "peak": peak, "unit": "GB/s", "frac": dom["gbs"] / peak,
                  "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks
                  else "fallback 6.8 TB/s",
                  "algorithmic": "lower triangle of the trailing matrix per column, read once (FP32 complex): "
                                 "N^3/6 elements x 8 B per matrix"})
        tr = profile_traffic(dom.get("ncu_name", ""))
        if tr:
            r["traffic"] = tr["bytes"]
            r["traffic_source"] = f"{tr['source']} ({tr['per']})"
        if "l2_read_gbs" in pipe:
            r["l2"] = {"peak_gbs": pipe["l2_read_gbs"], "frac": dom["gbs"] / pipe["l2_read_gbs"],
                       "peak_source": "live L2 read microbenchmark (nrltb_bench_peak kind 4)"}
        r["bound_note"] = ("the panel kernel's operands mostly stay in L2 (DRAM traffic well below the "
                           "algorithmic bytes); it is latency- and barrier-bound, so the fraction is also "
                           "given against the live L2 read bandwidth")
    elif dom["bound"] == "tensor":
        peak = peaks.get("bf16_tflops", 1900.0)
        r.update({"bound": "tensor", "achieved": dom["tflops"], "peak": peak, "unit": "TFLOP/s",
                  "frac": dom["tflops"] / peak,
                  "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS dense bf16, burst; of measured)",
                  "algorithmic": "8 flops per complex multiply-add the GEMM needs (triangular zeros and "
                                 "skipped C triangles excluded)"})
        tr = profile_traffic(dom.get("ncu_name", ""))
        if tr:
            r["traffic"] = tr["bytes"]
            r["traffic_source"] = f"{tr['source']} ({tr['per']})"
    else:
        kind = "fp64_fma_tflops" if prec == 0 else "fp32_fma_tflops"
        peak = pipe.get(kind)
        r.update({"bound": "tensor", "achieved": dom["tflops"], "peak": peak, "unit": "TFLOP/s",
                  "frac": dom["tflops"] / peak if peak else None,
                  "peak_source": "live FMA-pipe microbenchmark (GB300 has no FP64 tensor path; "
                                 "MEASURED_PEAKS.json has no FMA-pipe figure)",
                  "algorithmic": "8 flops per complex multiply-add the GEMM needs"})
    r["pipe_peaks_live"] = pipe
    return r


def run_batch(args):
    """--config batch256: 256 structures of 4-64 atoms (spd and sp3 bases,
    N = 16-576) on 2^3-5^3 meshes through nrltb_bande_batch, one call per step
    (host buffers in and out: the batch entry point has no device-resident
    split, so value and e2e are the same call).  k-point solves/s over all
    structures' k points."""
    import ctypes as C
    import numpy as np
    import torch
    from nrltb import Context, Opts, abi, synth
    from nrltb.api import new_result
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    ctx = Context(local)
    items = synth.batch256()
    prec = {"fp64": abi.PREC_FP64}.get(args.precision, abi.PREC_MIXED)
    opts = [Opts(mode=4, precision=prec, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11) for (_, _, _, o) in items]
    n = len(items)
    cs = (abi.Structure_ * n)(*[it[0].to_c() for it in items])
    cp = (abi.Params_ * n)(*[it[1].to_c() for it in items])
    ck = (abi.KMesh_ * n)(*[it[2].to_c() for it in items])
    co = (abi.Opts_ * n)(*[op.to_c() for op in opts])
    made = [new_result(it[1].nv(it[0]), it[2].nk) for it in items]
    cr = (abi.Result_ * n)(*[m[0] for m in made])
    nsolve = sum(it[2].nk for it in items)
    nvs = [it[1].nv(it[0]) for it in items]

    def step():
        rc = ctx.lib.nrltb_bande_batch(ctx.h, n, cs, cp, ck, co, cr)
        if rc != 0:
            raise RuntimeError(ctx.lib.nrltb_last_error().decode())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / args.steps
    launches = ctx.launch_count() - l0
    value = nsolve / (ms * 1e-3)
    h2d = sum(it[0].kkind.nbytes + it[0].posn.nbytes + it[0].posq.nbytes + it[1].param.nbytes + it[2].k.nbytes +
              it[2].w.nbytes for it in items)
    d2h = sum(m[1]["eig"].nbytes + m[1]["deig"].nbytes + m[1]["ncut"].nbytes + m[1]["k_status"].nbytes + 64
              for m in made)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == abi.PREC_FP64 else "f32+f64",
            "data": "synthetic (seeded structures and parameters, no public dataset)",
            "config": {"workload": f"batch256: {n} structures, 4-64 atoms, N = {min(nvs)}-{max(nvs)}, "
                                   f"{nsolve} k-point solves per step, mode 4, one nrltb_bande_batch call",
                       "precision": "fp64" if prec == abi.PREC_FP64 else "mixed",
                       "l2": "each step's matrices and workspace (GBs over the batch) exceed L2"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "note": "the batch entry point takes host buffers: value is this end-to-end call"},
            "gpu_launches": int(launches), "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        # the oracle on a bounded sample: the first 8 structures, all host cores
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        ncores = host_cores()
        t0 = time.perf_counter()
        ns = 0
        for (st, par, km, o), op in list(zip(items, opts))[:8]:
            oracle.bande(st, par, km, Opts(mode=4, tkb=o["tkb"], eigcut=1e3), nthreads=ncores)
            ns += km.nk
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": ns / t, "unit": UNIT, "cores": ncores, "kind": "port",
                                "sample": f"the first 8 structures of the batch ({ns} k-point solves), "
                                          f"one k per host thread"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="fcc128")
    ap.add_argument("--row", default="path", choices=ROWS)
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-form timing of the same step")
    ap.add_argument("--fp64-steps", type=int, default=2, help="timed steps of the FP64 form (after one untimed)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "batch256":
        return run_batch(args)

    import numpy as np
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from nrltb import Context, Opts, abi
    ctx = Context(local)
    lib = ctx.lib
    st0, par0, km, o = workload(args.config)
    st, par, mode, flags, per_k = row_setup(args.row, st0, par0)
    nk = km.nk * per_k   # solves per step: k points times spin channels
    prec = {"fp64": abi.PREC_FP64, "mixed": abi.PREC_MIXED}.get(args.precision)
    if prec is None:
        prec = abi.PREC_MIXED if _mixed_available(ctx, st0, par0, km) else abi.PREC_FP64
    opts = Opts(mode=mode, precision=prec, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11, flags=flags)

    stream = torch.cuda.Stream(local)
    ctx.set_stream(stream.cuda_stream)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    def max_over_ranks(x):
        if ws == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    # ---- device-resident value ----
    ctx.stage(st, par, km, opts)
    for _ in range(args.warmup):
        ctx.run()
    barrier()
    l0 = ctx.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            ctx.run()
        e1.record(stream)
        barrier()
    launches_value = ctx.launch_count() - l0
    # the same K steps again with per-class CUDA events around every launch of
    # the timed classes (kept out of the region `value` comes from)
    lib.nrltb_bench_kernel_timing(ctx.h, 1)
    for _ in range(args.steps):
        ctx.run()
    barrier()
    lib.nrltb_bench_kernel_timing(ctx.h, 0)
    kernels = kernel_stats(lib, ctx, args.steps)
    ms_dev = e0.elapsed_time(e1) / args.steps
    ms_dev = max_over_ranks(ms_dev)
    clocks = clk.summary()
    res = ctx.fetch()
    value = ws * nk / (ms_dev * 1e-3)

    # ---- end to end through nrltb_bande with host buffers ----
    for _ in range(2):
        ctx.bande(st, par, km, opts)
    barrier()
    l1 = ctx.launch_count()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        r = ctx.bande(st, par, km, opts)
    e1.record(stream)
    barrier()
    ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps)
    launches_e2e = ctx.launch_count() - l1
    e2e_value = ws * nk / (ms_e2e * 1e-3)
    h2d = ((st.spinat.nbytes if st.spinat is not None else 0) +
           st.kkind.nbytes + st.posn.nbytes + st.posq.nbytes + par.kbas.nbytes + par.dnn.nbytes +
           par.screenl.nbytes + par.param.nbytes + km.k.nbytes + km.w.nbytes + 8 * 3 * st.natoms)
    d2h = r.eig.nbytes + r.deig.nbytes + r.ncut.nbytes + r.k_status.nbytes + 64
    if r.orbocc is not None:
        d2h += r.orbocc.nbytes

    # ---- the FP64 form on the same step (the metric's other half) ----
    fp64 = None
    if prec == abi.PREC_MIXED and not args.no_fp64:
        opts64 = Opts(mode=mode, precision=abi.PREC_FP64, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11, flags=flags)
        ctx.stage(st, par, km, opts64)
        ctx.run()                                   # one untimed step (buffers sized, clocks up)
        k64 = max(1, min(args.steps, args.fp64_steps))
        barrier()
        e0.record(stream)
        for _ in range(k64):
            ctx.run()
        e1.record(stream)
        barrier()
        ms64 = max_over_ranks(e0.elapsed_time(e1) / k64)
        r64 = ctx.fetch()
        fp64 = {"value": ws * nk / (ms64 * 1e-3), "unit": UNIT, "ms_per_step": ms64, "steps": k64,
                "warmup": 1, "dtype": "f64"}
        # accuracy of the mixed form against the FP64 GPU form, every k point
        # of the step (outside any timed region)
        ok = (res.k_status == 0) & (r64.k_status == 0)
        fp64["mixed_vs_fp64"] = {
            "k_points_compared": int(ok.sum()),
            "max_abs_eig_ry": float(np.abs(res.eig[ok] - r64.eig[ok]).max()) if ok.any() else None,
            "abs_efermi_ry": abs(res.efermi - r64.efermi),
            "abs_etotal_ry_per_atom": abs(res.e_total - r64.e_total) / st.natoms,
            "abs_pressure_kbar": abs(res.pressure - r64.pressure) * 147105.08,
            "tolerances": {"eig_ry": 1e-9, "efermi_ry": 1e-9, "etotal_ry_per_atom": 1e-8, "pressure_kbar": 1e-3}}

    # ---- roofline of the dominant kernel class, from the timed region's events ----
    pipe = pipe_peaks(lib, ctx)
    roofline = roofline_of(kernels, prec, pipe)
    # whole-eigensolve figure: F_eig(N) = 24 N^3 real flops per k-point solve
    nv = int(res.nv)
    eig_tflops = value * 24.0 * nv ** 3 / 1e12
    peaks = measured_peaks()
    tf32 = peaks.get("bf16_tflops", 1900.0) / 2.0
    eigensolve = {"flops_per_solve": 24.0 * nv ** 3, "achieved_tflops": eig_tflops,
                  "tf32_peak_tflops": tf32, "frac": eig_tflops / tf32,
                  "peak_source": "half of MEASURED_PEAKS.json bf16_tflops (TF32 runs at half the bf16 rate "
                                 "on the tcgen05 tensor cores; no measured TF32 figure)",
                  "note": "k-point solves/s x 24 N^3, the complex LAPACK operation count of one generalized "
                          "eigensolve with vectors"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_dev, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == abi.PREC_FP64 else "f32+f64",
            "data": "synthetic (seeded structure and parameters, no public dataset)",
            "config": {"workload": workload_desc(args.config, st0, par0, km, args.row),
                       "precision": "fp64" if prec == abi.PREC_FP64 else "mixed",
                       "l2": "inputs larger than L2 (H,S,dH,dS + workspace of 27 k are GBs)",
                       "E_F": res.efermi, "E_total": res.e_total, "P": res.pressure},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e},
            "gpu_launches": int(launches_value),
            "gpu_launches_e2e": int(launches_e2e),
            "clocks": clocks, "roofline": roofline, "eigensolve_roofline": eigensolve, "kernels": kernels}
    if fp64 is not None:
        line["fp64"] = fp64
        line["fp64_value"] = fp64["value"]
        line["mixed_over_fp64"] = value / fp64["value"]

    if rank == 0 and not args.no_cpu_baseline:
        ncores = host_cores()
        nks = min(km.nk, ncores)
        t, ro = cpu_sample(st, par, km, mode, ncores, nks, flags)
        line["cpu_baseline"] = {"value": per_k * nks / t, "unit": UNIT, "cores": ncores, "kind": "port",
                                "sample": f"{nks} of {km.nk} k points, one per host thread, mode {mode} "
                                          f"(setham + zhpgv with vectors + sethamv + perturb + Fermi/E/P)",
                                "cores_note": "the host cores this process may run on (its affinity mask)"}
        if args.row == "path":
            # the same k points' eigenvalues from the GPU step against the oracle's
            rows = np.arange(nks)
            ok = res.k_status[rows] == 0
            line["accuracy_vs_oracle"] = {
                "k_points": int(ok.sum()), "form": "mixed" if prec == abi.PREC_MIXED else "fp64",
                "max_abs_eig_ry": float(np.abs(res.eig[rows][ok] - ro.eig[ok]).max()) if ok.any() else None}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def _mixed_available(ctx, st, par, km):
    from nrltb import abi
    import ctypes as C
    import numpy as np
    # a 1x1 probe: the mixed form reports NRLTB_E_UNSUPPORTED when it is not built
    H = np.array([[[2.0 + 0j]]])
    S = np.array([[[1.0 + 0j]]])
    eig = np.zeros((1, 1))
    stv = np.zeros(1, np.int32)
    rc = ctx.lib.nrltb_diag(ctx.h, 1, 1, H.ctypes.data_as(abi._dp), S.ctypes.data_as(abi._dp), abi.PREC_MIXED,
                            eig.ctypes.data_as(abi._dp), None, stv.ctypes.data_as(C.POINTER(C.c_int)))
    return rc == 0


if __name__ == "__main__":
    sys.exit(main())
