"""Run one small per-structure k loop, for profiling a kernel on a small case.

    python -m nrltb.profile_case --config fcc128 --nk 2 --precision mixed

runs nrltb_bande once on the first `nk` k points of a synthetic configuration
(after one untimed warm-up call), so that a profiler capture sees few launches
and a device footprint of a few hundred MB.
"""
import argparse
import time

import numpy as np

from . import Context, KMesh, Opts, abi, synth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="fcc128", choices=sorted(synth.CONFIGS))
    ap.add_argument("--nk", type=int, default=2)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--mode", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=1)
    args = ap.parse_args()
    st, par, km, o = synth.CONFIGS[args.config]()
    nk = min(args.nk, km.nk)
    sub = KMesh(km.k[:nk], np.full(nk, 1.0 / nk))
    prec = abi.PREC_FP64 if args.precision == "fp64" else abi.PREC_MIXED
    opts = Opts(mode=args.mode, precision=prec, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11)
    ctx = Context(0)
    for _ in range(args.warmup):
        ctx.bande(st, par, sub, opts)
    t0 = time.perf_counter()
    r = ctx.bande(st, par, sub, opts)
    dt = time.perf_counter() - t0
    print(f"{args.config} N={par.nv(st)} nk={nk} {args.precision}: {dt * 1e3:.1f} ms, "
          f"E_F={r.efermi:.12f} launches={ctx.launch_count()}")
    ctx.close()


if __name__ == "__main__":
    main()
