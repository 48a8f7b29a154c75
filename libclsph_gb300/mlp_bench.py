"""Times the stepper network's fused inference kernels on random rows.

    python -m libclsph_gb300.mlp_bench [--rows 1048576] [--iters 20] [--warmup 3]

Prints one JSON line: milliseconds per launch and FLOP/s of the tcgen05
kernel (clsph_mlp_forward) and of the mma.sync cross-check
(clsph_mlp_forward_mma_sync), with the fraction of the measured BF16 tensor
peak (MEASURED_PEAKS.json at the repository root, when present). FLOPs count
2 per multiply-add of the three layers: 2 * rows * (32*256 + 256*256 + 256*4).
Device buffers are torch tensors (plain device memory).
"""

from __future__ import annotations

import argparse
import json
from pathlib import Path

import numpy as np

from . import learned as Lm


def main(argv=None) -> dict:
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=1 << 20)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--weights", default=None, help="blob file (default: random weights)")
    args = ap.parse_args(argv)
    torch.cuda.set_device(0)
    if args.weights:
        net = Lm.Mlp.load(args.weights)
    else:
        blob = np.zeros(Lm.BLOB, np.float32)
        rng = np.random.default_rng(0)
        blob[:Lm.N_PARAMS] = rng.normal(0, 0.05, Lm.N_PARAMS)
        blob[Lm.OFF_XSIGMA:Lm.OFF_YMU] = 1
        blob[Lm.OFF_YSIGMA:] = 1
        net = Lm.Mlp(blob=blob)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(args.rows, Lm.N_FEATURES, device="cuda", generator=g).to(torch.bfloat16)
    y = torch.empty(args.rows, Lm.N_OUTPUTS, device="cuda")
    flops = 2.0 * args.rows * (32 * 256 + 256 * 256 + 256 * 4)
    out = {"rows": args.rows, "iters": args.iters, "flop_per_launch": flops}
    peak = None
    peaks = Path(__file__).resolve().parent.parent / "MEASURED_PEAKS.json"
    if peaks.exists():
        peak = json.loads(peaks.read_text()).get("bf16_tflops")
    for name, fn in (("tcgen05", net.forward), ("mma_sync", net.forward_mma_sync)):
        for _ in range(args.warmup):
            fn(x.data_ptr(), args.rows, y.data_ptr())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.iters):
            fn(x.data_ptr(), args.rows, y.data_ptr())
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.iters
        tf = flops / ms / 1e9
        out[name] = {"ms": ms, "tflops": tf, "frac_of_measured_bf16_peak": tf / peak if peak else None}
    out["status"] = net.status()
    net.close()
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
