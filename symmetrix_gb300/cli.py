"""Command-line utilities for the GB300 engine.

    python -m symmetrix_gb300.cli gen-model --config fp32_4096 --seed 1 --zbl out.json
    python -m symmetrix_gb300.cli eval --model out.json --atoms 4096 --density 0.10 --evals 3 [--precision bfloat16]
                                       [--option KEY=VALUE ...]

    python -m symmetrix_gb300.cli cache model.json model.smxb

`gen-model` writes a seeded synthetic model in libsymmetrix's JSON format;
`eval` builds a seeded random periodic box of the model's species and runs E+F
evaluations of it through the device-pointer C ABI (the call a GPU-resident caller
makes), printing per-evaluation device times.  `cache` writes the binary model cache
that MACE() (smx_create) loads without parsing the JSON.  `eval` is also the small, fixed target
used for ncu captures of single kernels; --option sets engine options (smx_set_option)
before the first evaluation, e.g. autotune=0 for a fixed schedule without tuning launches.
"""
import argparse
import json
import os
import sys
import time

import numpy as np


def gen_model(args):
    from .synth.model import CONFIGS, make_model, write_model
    cfg = dict(CONFIGS[args.config])
    if args.knots:
        cfg["num_knots"] = args.knots
    t = time.time()
    write_model(make_model(**cfg, seed=args.seed, zbl=args.zbl), args.out)
    print(f"wrote {args.out} ({os.path.getsize(args.out) / 1e6:.1f} MB) in {time.time() - t:.1f} s")


def evaluate(args):
    from . import MACE
    from .build import build
    from .synth.structures import neighbor_list, random_box

    build()
    eng = MACE(args.model, device=args.device, precision=args.precision)
    for kv in args.option:
        k, v = kv.split("=", 1)
        eng.set_option(k, int(v))
    pos, L, species = random_box(args.atoms, args.density, args.min_dist, eng.num_elements, seed=args.seed)
    nl = neighbor_list(pos, eng.r_cut, L)
    N, E = args.atoms, len(nl["r"])
    import torch  # device buffers for the inputs and outputs
    dev = torch.device("cuda", args.device)
    t = [torch.as_tensor(species, dtype=torch.int32, device=dev),
         torch.as_tensor(nl["num_neigh"], dtype=torch.int32, device=dev),
         torch.as_tensor(nl["neigh_indices"], dtype=torch.int32, device=dev),
         torch.as_tensor(species[nl["neigh_indices"]], dtype=torch.int32, device=dev),
         torch.as_tensor(nl["xyz"].reshape(-1), dtype=torch.float64, device=dev),
         torch.as_tensor(nl["r"], dtype=torch.float64, device=dev)]
    e_out = torch.zeros(N, dtype=torch.float64, device=dev)
    f_out = torch.zeros(3 * E, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    times = []
    with torch.cuda.stream(stream):
        for k in range(args.evals):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.compute_device(N, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), E,
                               t[4].data_ptr(), t[5].data_ptr(), e_out.data_ptr(), f_out.data_ptr(),
                               stream.cuda_stream)
            b.record(stream)
            times.append((a, b))
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in times]
    print(json.dumps({"atoms": N, "edges": E, "ms_per_eval": ms, "energy": float(e_out.sum().item())}))


def cache(args):
    from . import save_model_cache
    from .build import build
    build()
    t = time.time()
    save_model_cache(args.model, args.out)
    print(f"wrote {args.out} ({os.path.getsize(args.out) / 1e6:.1f} MB) in {time.time() - t:.1f} s")


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m symmetrix_gb300.cli")
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("gen-model")
    g.add_argument("out")
    g.add_argument("--config", default="fp32_4096")
    g.add_argument("--seed", type=int, default=1)
    g.add_argument("--knots", type=int, default=0)
    g.add_argument("--zbl", action="store_true")
    e = sub.add_parser("eval")
    e.add_argument("--model", required=True)
    e.add_argument("--atoms", type=int, default=4096)
    e.add_argument("--density", type=float, default=0.10)
    e.add_argument("--min-dist", type=float, default=0.9)
    e.add_argument("--seed", type=int, default=2)
    e.add_argument("--evals", type=int, default=3)
    e.add_argument("--device", type=int, default=0)
    e.add_argument("--precision", default="float32", choices=["float32", "bfloat16"])
    e.add_argument("--option", action="append", default=[], help="engine option KEY=VALUE (repeatable)")
    c = sub.add_parser("cache")
    c.add_argument("model")
    c.add_argument("out")
    args = ap.parse_args(argv)
    if args.cmd == "gen-model":
        gen_model(args)
    elif args.cmd == "cache":
        cache(args)
    else:
        evaluate(args)


if __name__ == "__main__":
    main()
