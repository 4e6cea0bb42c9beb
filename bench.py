#!/usr/bin/env python3
"""Throughput of the GB300 MACE engine on the 4096-atom workload, BF16-mixed vs FP32.

Workload (the single-GPU configuration the headline metric is quoted on): a
periodic cubic box of 4096 atoms at 0.10 atoms/A^3 (H/C/N/O uniform, minimum pair
distance 0.9 A, seeded random insertion) with a seeded random 2-layer MACE of
128x0e+128x1o channels, l_max 3, correlation 3, r_cut 5 A, 8 Bessel radials with
p=5 envelope tabulated on 200 spline knots.  Synthetic data: no public dataset or
checkpoint is involved.

The model has no ZBL pair repulsion and no density normalisation, as the
configuration states.

A step is one velocity-Verlet MD step of the whole box (dt 0.5 fs, Maxwell-Boltzmann
velocities at 300 K): edge geometry, the full E+F evaluation (forward and adjoint
pass), scatter to atomic forces and both half-kicks, with the neighbour list
(r_cut + 1 A skin) rebuilt on the GPU every 10 steps; the steps between rebuilds run
as one captured CUDA graph.  `value` is atoms x steps / device time (CUDA events on
the engine's stream).  No L2 flush between steps: the working set of a step (spline
tables, node features and adjoints, edge arrays) is several times the 129 MB L2.
Both forms run the same MD: `value` is the BF16-mixed form (channel-mixing GEMMs on
the tcgen05 tensor cores with bf16 split operands), `forms` holds both forms'
throughput and their energy / force / virial errors against the float64 oracle on
the timed structure itself (the full box; for the 32768- and 1,048,576-atom shapes a
4096-atom box of the same model, density and species mix, and with --full-check the
whole 32768-atom box).  The CPU baseline is the same float64 oracle evaluating that
structure on all host threads (and one thread on a 256-atom box).
`e2e` is the same metric through the host-pointer C ABI evaluator call a LAMMPS/ASE
caller makes every step (host->device copy of the neighbour list and device->host
copy of energies and forces inside the timed region).  Per-kernel times for the
roofline come from engine CUDA events over a separate pass of evaluation steps on
the same structure, with L2 flushed between those steps.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                       [--workload fp32_4096|precision_32768|large_1m|molecules|pair_modes]
                       [--detail PATH] [--full-check]
--detail writes the long form of the result (per-stage FLOP and byte rates, MD energy
record, schedules) to PATH; stdout carries one compact line.
Multi-GPU (torchrun): every rank evaluates its own replica of the box (the
engine does not shard one box over GPUs); value is the job's total.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "atom-steps/s (E+F) on 1 GB300: BF16-mixed vs FP32 at <=10 meV/A force error"
UNIT = "atom-steps/s"
WORKLOADS = {
    # the headline: 4096 atoms, 128x0e+128x1o, H/C/N/O, r_cut 5
    "fp32_4096": dict(name="fp32_4096", config="fp32_4096", n_atoms=4096, density=0.10, min_dist=0.9, n_species=4,
                      r_cut=5.0, model_seed=1, struct_seed=2, cpu_sample_atoms=256, err_atoms=None,
                      text="fp32_4096: periodic box, 4096 atoms, 0.10 atoms/A^3, H/C/N/O, 128x0e+128x1o, l_max 3, "
                           "correlation 3, r_cut 5 A, 200 spline knots"),
    # the precision-form shape: 32768 atoms, 128x0e+128x1o+128x2e, 10 species, r_cut 6
    # the large single system: 1,048,576 atoms, 128x0e+128x1o, 10 species, r_cut 5 (MD only)
    "large_1m": dict(name="large_1m", config="large_1m", n_atoms=1048576, density=0.10, min_dist=0.9, n_species=10,
                     r_cut=5.0, model_seed=1, struct_seed=2, cpu_sample_atoms=128, err_atoms=4096,
                     text="large_1m: periodic box, 1,048,576 atoms, 0.10 atoms/A^3, 10 species, 128x0e+128x1o, "
                          "l_max 3, correlation 3, r_cut 5 A, 200 spline knots"),
    "precision_32768": dict(name="precision_32768", config="bf16_32768", n_atoms=32768, density=0.09, min_dist=0.9,
                            n_species=10, r_cut=6.0, model_seed=1, struct_seed=2, cpu_sample_atoms=128,
                            err_atoms=4096,
                            text="precision_32768: periodic box, 32768 atoms, 0.09 atoms/A^3, 10 species, "
                                 "128x0e+128x1o+128x2e (L_max 2), l_max 3, correlation 3, r_cut 6 A, 200 spline "
                                 "knots"),
}
WORKLOAD = WORKLOADS["fp32_4096"]
CACHE = os.path.join(tempfile.gettempdir(), "smx_bench")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def model_path():
    from symmetrix_gb300.synth.model import CONFIGS, make_model, write_model
    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, f"model_{WORKLOAD['name']}_s{WORKLOAD['model_seed']}.json")
    if not os.path.exists(path):
        t = time.time()
        model = make_model(**CONFIGS[WORKLOAD["config"]], seed=WORKLOAD["model_seed"])
        json.dump(dims_of(model), open(path + ".dims.json", "w"))
        write_model(model, path + ".tmp")
        del model
        os.replace(path + ".tmp", path)
        log(f"model written in {time.time() - t:.1f} s")
    return path


def engine_model_path(path):
    """The engine loads a binary cache of the model (written once next to the JSON)."""
    from symmetrix_gb300 import save_model_cache
    cache = path[:-5] + ".smxb"
    if not os.path.exists(cache):
        save_model_cache(path, cache + ".tmp")
        os.replace(cache + ".tmp", cache)
    return cache


def structure(n_atoms, seed):
    from symmetrix_gb300.synth.structures import neighbor_list, random_box
    pos, L, species = random_box(n_atoms, WORKLOAD["density"], WORKLOAD["min_dist"], WORKLOAD["n_species"], seed=seed)
    nl = neighbor_list(pos, WORKLOAD["r_cut"], L)
    return pos, L, species, nl


def model_dims(eng, path):
    dims_path = path + ".dims.json"
    if os.path.exists(dims_path):
        return json.load(open(dims_path))
    with open(path) as f:
        m = json.load(f)
    d = dims_of(m)
    json.dump(d, open(dims_path, "w"))
    return d


def dims_of(m):
    C = m["num_channels"]
    L_max = m["L_max"]
    n_e = [sum(1 for l in m["Phi1_l"] if l == ll) for ll in range(4)]
    return dict(C=C, S=m["num_elements"], nLM=(L_max + 1) ** 2, n_lme=sum((2 * l + 1) for l in m["Phi1_l"]),
                NI=len(m["Phi1_l"]), NP=sum((2 * a + 1) * (2 * b + 1) for a, b in zip(m["Phi1_l1"], m["Phi1_l2"])),
                G=len(m["Phi1_clebsch_gordan"]), T0=[len(m["M0_monomials"][str(q)]) for q in range((L_max + 1) ** 2)],
                T1=len(m["M1_monomials"]), nint=len(m["radial_spline_values_0"][0][0]) - 1,
                npairs=len(m["radial_spline_values_0"]), n_e=n_e, nh=len(m["readout_2_weights_2"]),
                l1=m["Phi1_l1"], l2=m["Phi1_l2"])


def stage_costs(d, N, E):
    """Algorithmic FLOPs and compulsory DRAM bytes of each kernel launch (FP32 storage)."""
    C, S, nLM, n_lme, NI, NP, G = d["C"], d["S"], d["nLM"], d["n_lme"], d["NI"], d["NP"], d["G"]
    f4 = 4
    spl0 = S * S * d["nint"] * 4 * C * 16
    spl1 = d["npairs"] * d["nint"] * NI * C * 16
    coef0 = S * sum(d["T0"]) * C * f4
    sum_2l1 = sum(2 * a + 1 for a in d["l1"])
    out = {}
    out["layer0_fwd"] = (E * C * 56 + N * C * 4 * sum(d["T0"]),
                         E * 36 + 8 * N + spl0 + coef0 + N * (16 + nLM) * C * f4)
    out["gemm_H1"] = (2 * N * nLM * C * C, 2 * N * nLM * C * f4 + nLM * C * C * f4)
    out["layer1_fwd"] = (E * C * (6 * NI + sum_2l1 + 2 * NP) + 2 * N * C * G,
                         E * 40 + 8 * N + N * nLM * C * f4 + spl1 + N * n_lme * C * f4)
    out["gemm_A1"] = (2 * N * C * C * n_lme, N * (n_lme + 16) * C * f4 + n_lme * C * C * f4)
    out["node_tail"] = (N * C * (10 * d["T1"] + 8 * C + 4 * d["nh"]),
                        N * (16 + 1) * C * f4 + N * (4 + 16 + nLM) * C * f4 + 8 * N + (2 * S + 2) * C * C * f4)
    out["gemm_Phi1_adj"] = (2 * N * C * C * n_lme, N * (n_lme + 16) * C * f4 + n_lme * C * C * f4)
    out["layer1_rev"] = (E * C * (10 * NI + 4 * NP + 5 * sum_2l1 + 2 * NI + 102) + 2 * N * C * G,
                         E * 52 + 8 * N + N * (n_lme + nLM) * C * f4 + spl1 + 2 * N * nLM * C * f4)
    out["gemm_M0_adj"] = (2 * N * nLM * C * C, 2 * N * nLM * C * f4 + nLM * C * C * f4)
    out["layer0_rev"] = (E * C * (40 + 16 * 9 + 14) + N * C * 10 * sum(d["T0"]),
                         E * (36 + 12 + 24) + 8 * N + spl0 + coef0 + N * (16 + nLM) * C * f4)
    return out


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"smx_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# the float64 oracle: the error reference and the CPU baseline
# ---------------------------------------------------------------------------
def host_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def edge_tuple(species, nl):
    return (len(species), species, nl["num_neigh"], nl["neigh_indices"], species[nl["neigh_indices"]], nl["xyz"],
            nl["r"])


def sig(x, n=4):
    """x rounded to n significant digits (keeps the JSON line short)."""
    return float(f"{x:.{n}g}") if x is not None else None


def oracle_eval(path, a, threads, repeats=0, lean=None):
    """The float64 oracle's result for one structure, evaluated on `threads` host threads
    (each stage split over node ranges, bitwise equal to one thread), and with repeats > 0
    the median time of `repeats` evaluations after one warm-up.  The radials are stored per
    edge as the reference does unless that would take more than 16 GB (lean)."""
    from oracle.pyoracle import Evaluator
    ev = Evaluator(path, "port").set_threads(threads)
    if lean is None:
        lean = len(a[6]) * ev.num_channels * 17 * 16 > 16e9
    ev.set_lean(lean)
    times = []
    for _ in range(repeats + 1):
        t = time.perf_counter()
        ev.compute_node_energies_forces(*a)
        times.append(time.perf_counter() - t)
    ref = {"node_energies": np.array(ev.node_energies), "node_forces": np.array(ev.node_forces)}
    return ref, (statistics.median(times[1:]) if repeats > 0 else times[0])


def errors(e, f, ref, nl):
    """Energy, force and virial errors of GPU outputs (node energies, per-edge forces)
    against the float64 oracle's for the same structure."""
    n = len(e)
    f = np.asarray(f).reshape(-1, 3)
    fr = ref["node_forces"].reshape(-1, 3)
    er = ref["node_energies"]

    def atomic(fe):
        F = np.zeros((n, 3))
        np.add.at(F, nl["i"], -fe)
        np.add.at(F, nl["neigh_indices"], fe)
        return F

    def virial(fe):  # W_ab = -sum_e x_a f_b over directed edges (force on j from edge i->j is f)
        x = nl["xyz"].reshape(-1, 3)
        return -(x[:, :, None] * fe[:, None, :]).sum(0)

    dF = np.abs(atomic(f) - atomic(fr))
    return {"energy_per_atom_eV": sig(abs(np.sum(e) - er.sum()) / n, 3),
            "max_node_energy_eV": sig(float(np.abs(np.asarray(e) - er).max()), 3),
            "max_force_eV_per_A": sig(float(dF.max()), 3), "rms_force_eV_per_A": sig(float(np.sqrt((dF ** 2).mean())), 3),
            "max_edge_force_eV_per_A": sig(float(np.abs(f - fr).max()), 3),
            "max_virial_eV": sig(float(np.abs(virial(f) - virial(fr)).max()), 3)}


def cpu_model():
    """The host CPU as /proc/cpuinfo names it (model name, or implementer/part on Arm)."""
    import platform
    fields = {}
    try:
        for line in open("/proc/cpuinfo"):
            if ":" in line:
                k, v = (x.strip() for x in line.split(":", 1))
                fields.setdefault(k, v)
    except OSError:
        pass
    name = fields.get("model name") or " ".join(f"{k} {fields[k]}" for k in ("CPU implementer", "CPU part")
                                                if k in fields)
    return f"{platform.machine()} {name}".strip()


def reference_arm(args, rank, world):
    """The CPU path: the float64 oracle (restatement of libsymmetrix/source/mace.cpp)
    evaluating the GPU arm's structure on all host threads, one evaluation per step."""
    if rank != 0:
        return
    path = model_path()
    threads = host_threads()
    n = WORKLOAD["err_atoms"] or WORKLOAD["n_atoms"]
    full = n == WORKLOAD["n_atoms"]
    pos, L, species, nl = structure(n, WORKLOAD["struct_seed"] + (0 if full else 100))
    from oracle.pyoracle import Evaluator
    ev = Evaluator(path, "port").set_threads(threads)
    a = edge_tuple(species, nl)
    for _ in range(args.warmup):
        ev.compute_node_energies_forces(*a)
    t = time.perf_counter()
    for _ in range(args.steps):
        ev.compute_node_energies_forces(*a)
    dt = (time.perf_counter() - t) / args.steps
    value = n / dt
    sample = (f"one E+F evaluation per step of the {n}-atom box " + ("the GPU arm times" if full else
              "of the same model, density and species mix") + f" ({len(nl['r'])} edges), float64 oracle "
              f"restatement of libsymmetrix/source/mace.cpp, each stage split over {threads} host threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD["name"], "atoms_per_step": n, "threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "cpu": cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def time_md(eng, pos, species, masses, L, vel, args, dist, estream):
    """The timed region: `args.steps` MD steps after `args.warmup` untimed ones."""
    import torch

    from symmetrix_gb300.md import MD
    N = len(species)
    md = MD(eng, pos, species, masses, box=L, velocities=vel, dt=0.5, skin=1.0, rebuild_every=10)
    st0 = md.state()
    md.run(args.warmup)
    md.sync()
    stw = md.state()
    if dist:
        dist.barrier()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    e0.record(estream)
    md.run(args.steps)
    e1.record(estream)
    md.sync()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    if dist:
        dist.barrier()
    clk = clocks.stop()
    T = e0.elapsed_time(e1) / 1e3
    if dist:
        tt = torch.tensor([T], device=torch.device("cuda", torch.cuda.current_device()))
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        T = tt.item()
    st1 = md.state()
    acc = 9.648533212331e-3
    ke = lambda v: 0.5 * float((masses[:, None] * v ** 2).sum()) / acc
    kelvin = lambda v: 2 * ke(v) / (3 * N * 8.617333262e-5)
    md_check = {"E_total_start": st0["potential_energy"] + ke(st0["velocities"]),
                "E_total_after_warmup": stw["potential_energy"] + ke(stw["velocities"]),
                "T_after_warmup_K": kelvin(stw["velocities"]),
                "E_total_end": st1["potential_energy"] + ke(st1["velocities"]),
                "T_end_K": kelvin(st1["velocities"]), "edges_skin_list": md.num_edges,
                "note": "random-weight synthetic potential (no short-range repulsion) on a random-insertion "
                        "box: forces of a few eV/A turn potential into kinetic energy from the first step, pairs "
                        "close to ~0.1 A within ~12 fs, and close encounters then break energy conservation at "
                        "dt 0.5 fs, so E_total_end and T_end_K of a long run say nothing about the integrator; "
                        "the per-step work (the skin-list edges) stays about the same"}
    del md
    return T, t_wall, clk, md_check


# (workload, stage) -> (DRAM bytes per launch, the ncu summary it comes from)
NCU_TRAFFIC = {
    ("fp32_4096", "layer1_rev"): (165.6e6 + 11.5e6, "profiles/layer1_rev_fp32_4096.md (ncu --set full, 1 launch)"),
}

ATOM_KERNELS = ("layer0_fwd", "contract0_rev", "layer0_rev", "layer1_fwd", "layer1_rev", "node_tail")


def schedule_of(eng):
    """The autotuned schedule the engine ran with: per-atom kernels on persistent grids, GEMM tiles."""
    mask = eng.get_option("persistent")
    out = {"persistent_kernels": [k for b, k in enumerate(ATOM_KERNELS) if mask >> b & 1],
           "species_order": eng.get_option("species_order"), "l2_channel_slices": eng.get_option("l2_split")}
    if eng.precision == "bfloat16":
        out["gemm"] = eng.gemm_schedule()
    return out


def stage_profile(eng, N, E, species, nl, n_prof, dev):
    """Per-stage device times (engine CUDA events) over n_prof evaluations, L2 flushed."""
    import torch
    eng.set_option("profile", 1)
    t_types = torch.as_tensor(species, dtype=torch.int32, device=dev)
    t_nn = torch.as_tensor(nl["num_neigh"], dtype=torch.int32, device=dev)
    t_idx = torch.as_tensor(nl["neigh_indices"], dtype=torch.int32, device=dev)
    t_nt = torch.as_tensor(species[nl["neigh_indices"]], dtype=torch.int32, device=dev)
    t_xyz = torch.as_tensor(nl["xyz"].reshape(-1), dtype=torch.float64, device=dev)
    t_r = torch.as_tensor(nl["r"], dtype=torch.float64, device=dev)
    t_e = torch.zeros(N, dtype=torch.float64, device=dev)
    t_f = torch.zeros(3 * E, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def eval_step():
        eng.compute_device(N, t_types.data_ptr(), t_nn.data_ptr(), t_idx.data_ptr(), t_nt.data_ptr(), E,
                           t_xyz.data_ptr(), t_r.data_ptr(), t_e.data_ptr(), t_f.data_ptr(), stream.cuda_stream)

    stage_tot, eval_ms = {}, []
    with torch.cuda.stream(stream):
        for _ in range(3):
            flush.fill_(1)
            eval_step()
        for k in range(n_prof):
            flush.fill_(k & 255)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eval_step()
            b.record(stream)
            for n_, v in eng.stage_times().items():
                stage_tot[n_] = stage_tot.get(n_, 0.0) + v
            eval_ms.append((a, b))
    torch.cuda.synchronize()
    eval_ms = [a.elapsed_time(b) for a, b in eval_ms]
    eng.set_option("profile", 0)
    return {n_: v / n_prof for n_, v in stage_tot.items()}, statistics.median(eval_ms)


def gpu_arm(args, rank, world, local_rank):
    import ctypes

    import torch

    from symmetrix_gb300 import MACE, _lib
    from symmetrix_gb300.build import build
    from symmetrix_gb300.synth.structures import maxwell_boltzmann, species_masses

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build()
    path = model_path()
    epath = engine_model_path(path)
    N = WORKLOAD["n_atoms"]
    pos, L, species, nl = structure(N, WORKLOAD["struct_seed"] + rank)
    E = len(nl["r"])
    dev = torch.device("cuda", local_rank)
    n_prof = max(5, min(args.steps, 20))

    # ---- both forms: MD timed region, per-stage times ----
    forms = {}
    for form in ("fp32", "bf16"):
        eng = MACE(epath, device=local_rank, precision=form)
        dims = model_dims(eng, path)
        estream = torch.cuda.ExternalStream(eng.stream, device=dev)
        masses = species_masses(eng.atomic_numbers, species)
        vel = maxwell_boltzmann(masses, 300.0, np.random.default_rng(WORKLOAD["struct_seed"] + rank))
        T, t_wall, clk, md_check = time_md(eng, pos, species, masses, L, vel, args, dist, estream)
        avg, eval_ms = stage_profile(eng, N, E, species, nl, n_prof, dev)
        forms[form] = {"eng": eng, "T": T, "t_wall": t_wall, "clk": clk, "md_check": md_check, "stages": avg,
                       "eval_ms": eval_ms, "value": world * N * args.steps / T, "schedule": schedule_of(eng)}
    head = forms["bf16"]
    eng = head["eng"]

    # ---- e2e: the host-pointer C ABI with pinned host buffers (headline form) ----
    lib = _lib.load()
    pin = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt).pin_memory()
    h = [pin(species, torch.int32), pin(nl["num_neigh"], torch.int32), pin(nl["neigh_indices"], torch.int32),
         pin(species[nl["neigh_indices"]], torch.int32), pin(nl["xyz"].reshape(-1), torch.float64),
         pin(nl["r"], torch.float64)]
    h_e = torch.zeros(N, dtype=torch.float64).pin_memory()
    h_f = torch.zeros(3 * E, dtype=torch.float64).pin_memory()
    P = lambda t: ctypes.c_void_p(t.data_ptr())

    def e2e_step():
        code = lib.smx_compute_node_energies_forces(eng._h, N, P(h[0]), P(h[1]), P(h[2]), P(h[3]), E, P(h[4]),
                                                    P(h[5]), P(h_e), P(h_f))
        _lib.raise_for(code, lib)

    for _ in range(args.warmup):
        e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    t_e2e = time.perf_counter() - t0
    if dist:
        tt = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = tt.item()
    e2e = {"value": world * N * args.steps / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": 4 * N + 4 * (N + 1) + E * (4 + 4 + 24 + 8), "d2h_bytes_per_step": 8 * N + 24 * E,
           "step": "one smx_compute_node_energies_forces call on host arrays (the pair-style call), BF16-mixed form"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ---- errors against the float64 oracle on the timed structure (or a 4096-atom box of
    # the same model for the larger shapes), and the CPU baseline on that structure ----
    threads = host_threads()
    err_n = WORKLOAD["err_atoms"] or N
    if err_n == N:
        nl_err, a_err = nl, edge_tuple(species, nl)
        err_box = f"the timed {N}-atom structure ({E} edges)"
    else:
        _, _, sp_e, nl_err = structure(err_n, WORKLOAD["struct_seed"] + 100)
        a_err = edge_tuple(sp_e, nl_err)
        err_box = f"a {err_n}-atom box of the same model, density and species mix ({len(nl_err['r'])} edges)"
    ref, t_cpu = oracle_eval(path, a_err, threads, repeats=3)
    errs = {"box": err_box}
    for name, form in forms.items():
        form["eng"].compute_node_energies_forces(*a_err)
        errs[name] = errors(form["eng"].node_energies, form["eng"].node_forces, ref, nl_err)
    del ref
    if args.full_check and err_n != N:  # the whole timed box against the oracle (lean radials)
        t = time.time()
        ref_full, _ = oracle_eval(path, edge_tuple(species, nl), threads, lean=True)
        errs_full = {"box": f"the timed {N}-atom structure ({E} edges)"}
        for name, form in forms.items():
            form["eng"].compute_node_energies_forces(*edge_tuple(species, nl))
            errs_full[name] = errors(form["eng"].node_energies, form["eng"].node_forces, ref_full, nl)
        del ref_full
        log(f"full-box oracle check in {time.time() - t:.0f} s")
    _, _, sp1, nl1 = structure(WORKLOAD["cpu_sample_atoms"], WORKLOAD["struct_seed"] + 100)
    _, t_one = oracle_eval(path, edge_tuple(sp1, nl1), 1, repeats=2)
    cpu = {"value": err_n / t_cpu, "unit": UNIT, "cores": threads, "kind": "port", "cpu": cpu_model(),
           "sample": f"median of 3 E+F evaluations after 1 warm-up of {err_box}, float64 oracle restatement of "
                     f"libsymmetrix/source/mace.cpp, each stage split over {threads} host threads",
           "single_core": {"value": sig(WORKLOAD["cpu_sample_atoms"] / t_one),
                           "sample": f"{WORKLOAD['cpu_sample_atoms']}-atom box, 1 thread, median of 2 after 1 "
                                     "warm-up"}}

    # ---- roofline of the dominant kernel (headline form) ----
    costs = stage_costs(dims, N, E)
    avg = head["stages"]
    dom = max(avg, key=avg.get)
    flops, bytes_ = costs[dom]
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peaks = json.load(open(peaks_path))
        hbm, peak_src = peaks["hbm_gbs"], "measured"
    else:
        hbm, peak_src = 6800.0, "fallback"
    t_dom = avg[dom] / 1e3
    achieved = bytes_ / t_dom / 1e9
    clk = head["clk"]
    sm_mhz = clk.get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    # DRAM bytes per launch of the dominant kernel from one ncu capture of this build
    # (dram__bytes_read.sum + dram__bytes_write.sum), where one exists for the workload
    traffic = NCU_TRAFFIC.get((WORKLOAD["name"], dom))
    roofline = {"bound": "hbm", "kernel": dom, "achieved": sig(achieved), "peak": hbm, "unit": "GB/s",
                "frac": sig(achieved / hbm), "peak_source": peak_src,
                "traffic": traffic[0] if traffic else None, "traffic_source": traffic[1] if traffic else None,
                "algorithmic_bytes_per_launch": bytes_, "avg_launch_ms": sig(avg[dom]),
                "fp32_simt": {"achieved_tflops": sig(flops / t_dom / 1e12), "peak_tflops": sig(fp32_peak),
                              "frac": sig(flops / t_dom / 1e12 / fp32_peak),
                              "peak_source": "152 SMs x 128 FP32 lanes x 2 x median SM clock under load"}}

    def per_stage(a):
        return {n_: {"ms": a[n_], "gflop": costs[n_][0] / 1e9, "tflops": costs[n_][0] / (a[n_] / 1e3) / 1e12,
                     "gbs": costs[n_][1] / (a[n_] / 1e3) / 1e9} for n_ in a}

    # kernels per MD step of the BF16 form: vv_first, edge geometry with the in-cut-off packing,
    # the atomic forces with the second half-kick, and 11 evaluation kernels (layer0_fwd,
    # layer1_fwd, node_tail, layer1_rev, contract0_rev, layer0_rev, four grouped tcgen05 GEMM
    # launches: H1, A1 (all l), Phi1_adj (all l), M0_adj, and the H1_adj rows' conversion to
    # the M0_adj GEMM's operand), one more when the centre atoms are species-sorted; plus per
    # rebuild: wrap, 4 cell-list kernels, the float copy of the positions, 2 neighbour passes,
    # scan, reverse map
    rebuilds = (args.warmup + args.steps + 9) // 10 - (args.warmup + 9) // 10
    per_step = 3 + 11 + (1 if eng.get_option("species_order") == 1 else 0)
    launches = per_step * args.steps + 10 * rebuilds
    fp = forms["fp32"]
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["T"] / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": WORKLOAD["text"], "atoms": N, "edges_r_cut": E,
                   "form": f"BF16-mixed: channel-mixing GEMMs on tcgen05, bf16 split operands "
                           f"({eng.get_option('tc_terms')} terms), f32 accumulation; radials, Y_lm, contractions, "
                           "adjoint f32; f64 sums",
                   "step": "velocity-Verlet MD step (E+F + integration); neighbour list rebuilt on the GPU every 10 "
                           "steps (1 A skin); CUDA graph between rebuilds",
                   "l2": "no flush: the per-step working set (>400 MB) exceeds L2", "replicas_per_gpu": 1},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "stages_ms": {"bf16": {n_: sig(v, 3) for n_, v in avg.items()},
                      "fp32": {n_: sig(v, 3) for n_, v in fp["stages"].items()}},
        "forms": {name: {"value": sig(f_["value"]), "ms_per_step": sig(f_["T"] / args.steps * 1e3),
                         "ms_per_eval": sig(f_["eval_ms"])} for name, f_ in forms.items()},
        "bf16_over_fp32": sig(head["value"] / fp["value"]),
        "errors_vs_fp64": errs,
    }
    if args.full_check and err_n != N:
        line["errors_vs_fp64_full_box"] = errs_full
    if args.detail:
        detail = dict(line)
        detail.update({"stages": {"bf16": per_stage(avg), "fp32": per_stage(fp["stages"])},
                       "md_check": {name: f_["md_check"] for name, f_ in forms.items()},
                       "schedule": {name: f_["schedule"] for name, f_ in forms.items()},
                       "clocks_fp32": fp["clk"], "wall_s_timed_region": head["t_wall"],
                       "eval_only": {"ms_per_eval": head["eval_ms"], "l2": "flushed between evaluations"}})
        with open(args.detail, "w") as fh:
            json.dump(detail, fh, indent=1)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# batching form (--workload molecules): not the headline line
# ---------------------------------------------------------------------------
MOLECULES = dict(name="molecules_2048", n_mol=2048, sizes=(8, 120), density=0.08, min_dist=0.95, seed=4,
                 species=("H", "C", "N", "O", "F", "S", "Cl"), probs=(0.45, 0.30, 0.08, 0.10, 0.03, 0.02, 0.02))


def molecule_reference(path, pos, sp, first, r_cut):
    """float64 oracle energies and atomic forces of every molecule (host threads over molecules)."""
    from oracle.pyoracle import Evaluator
    from symmetrix_gb300.synth.structures import neighbor_list
    n_mol = len(first) - 1
    threads = host_threads()
    base = Evaluator(path, "port")
    evs = [base] + [base.clone() for _ in range(threads - 1)]
    E_ref, F_ref = np.zeros(n_mol), [None] * n_mol

    def work(t):
        ev = evs[t]
        for m in range(t, n_mol, threads):
            p, s_ = pos[first[m]:first[m + 1]], sp[first[m]:first[m + 1]]
            nl = neighbor_list(p, r_cut)
            ev.compute_node_energies_forces(*edge_tuple(s_, nl))
            E_ref[m] = ev.node_energies.sum()
            f = ev.node_forces.reshape(-1, 3)
            F = np.zeros((len(p), 3))
            np.add.at(F, nl["neigh_indices"], f)
            np.add.at(F, nl["i"], -f)
            F_ref[m] = F

    t0 = time.time()
    ths = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    log(f"oracle over {n_mol} molecules in {time.time() - t0:.0f} s ({threads} threads)")
    return E_ref, F_ref


def molecule_errors(e_mol, F, ref, first):
    E_ref, F_ref = ref
    n = np.diff(first)
    dF = np.concatenate([np.abs(a - b) for a, b in zip(F, F_ref)])
    return {"box": f"all {len(n)} molecules ({int(n.sum())} atoms)",
            "energy_per_atom_eV": sig(abs(np.sum(e_mol) - E_ref.sum()) / n.sum(), 3),
            "max_molecule_energy_per_atom_eV": sig(float((np.abs(np.asarray(e_mol) - E_ref) / n).max()), 3),
            "max_force_eV_per_A": sig(float(dF.max()), 3), "rms_force_eV_per_A": sig(float(np.sqrt((dF ** 2).mean())), 3)}


def molecules_arm(args):
    import torch

    from symmetrix_gb300 import MACE
    from symmetrix_gb300.build import build
    from symmetrix_gb300.md import MD
    from symmetrix_gb300.synth.model import CONFIGS, make_model, write_model
    from symmetrix_gb300.synth.structures import maxwell_boltzmann, random_molecule, species_masses

    build()
    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, "model_molecules_s1.json")
    if not os.path.exists(path):
        write_model(make_model(**CONFIGS["molecules"], seed=1), path + ".tmp")
        os.replace(path + ".tmp", path)
    W = MOLECULES
    sfile = os.path.join(CACHE, f"{W['name']}_s{W['seed']}.npz")
    if os.path.exists(sfile):
        z = np.load(sfile)
        pos, sp, first = z["pos"], z["sp"], z["first"]
    else:
        rng = np.random.default_rng(W["seed"])
        P, S_, counts = [], [], []
        for m in range(W["n_mol"]):
            k = int(rng.integers(W["sizes"][0], W["sizes"][1] + 1))
            p, s_ = random_molecule(k, W["density"], W["min_dist"], len(W["species"]), rng, probs=W["probs"])
            # molecules on a 40 A grid (independence is by molecule, not by distance)
            P.append(p + 40.0 * np.array([m % 16, (m // 16) % 16, m // 256]))
            S_.append(s_)
            counts.append(k)
        pos, sp = np.concatenate(P), np.concatenate(S_).astype(np.int32)
        first = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        np.savez(sfile, pos=pos, sp=sp, first=first)
    N = len(pos)
    dev = torch.device("cuda", 0)
    out = {}
    ref = None
    for form in ("fp32", "bf16"):
        eng = MACE(path, precision=form)
        estream = torch.cuda.ExternalStream(eng.stream, device=dev)
        masses = species_masses(eng.atomic_numbers, sp)
        vel = maxwell_boltzmann(masses, 300.0, np.random.default_rng(7))
        md = MD(eng, pos, sp, masses, velocities=vel, dt=0.5, skin=1.0, rebuild_every=10, mol_first=first)
        md.run(args.warmup)
        md.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(estream)
        md.run(args.steps)
        e1.record(estream)
        md.sync()
        T = e0.elapsed_time(e1) / 1e3
        out[form] = {"value": N * args.steps / T, "ms_per_step": T / args.steps * 1e3, "edges": md.num_edges,
                     "schedule": schedule_of(eng)}
        del md
        # every molecule's energy and forces in one batched evaluation, against the oracle
        if ref is None:
            ref = molecule_reference(path, pos, sp, first, CONFIGS["molecules"]["r_cut"])
        e_mol, _, F = eng.compute_molecules([(pos[first[m]:first[m + 1]], sp[first[m]:first[m + 1]])
                                             for m in range(len(first) - 1)])
        out[form]["errors_vs_fp64"] = molecule_errors(e_mol, F, ref, first)
        del eng
    print(json.dumps({
        "metric": METRIC, "value": out["bf16"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": out["bf16"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": f"{W['name']}: {W['n_mol']} non-periodic molecules of {W['sizes'][0]}-{W['sizes'][1]} "
                               f"atoms ({N} atoms), 64x0e+64x1o, r_cut 5 A, H/C/N/O/F/S/Cl; batch MD, dt 0.5 fs, "
                               "neighbour list per molecule rebuilt every 10 steps, CUDA graph between rebuilds",
                   "atoms": N},
        "forms": out, "bf16_over_fp32": out["bf16"]["value"] / out["fp32"]["value"],
    }), flush=True)


# ---------------------------------------------------------------------------
# LAMMPS pair-style adapter (--workload pair_modes): not the headline line
# ---------------------------------------------------------------------------
def pair_modes_arm(args):
    """One compute() of pair_style symmetrix/mace per step, in each of its three modes,
    on the headline box laid out as one LAMMPS rank (4096 local atoms, ghost images
    2 r_cut + 1 A deep, full lists within r_cut + 1 A of every atom): host positions in,
    host forces, energy and virial out, timed on the host clock around the synchronous
    call (smx_pair_compute_mode).  Each mode's forces, folded onto the local atoms as
    LAMMPS's reverse communication does, are compared with the first mode's."""
    from symmetrix_gb300 import MACE
    from symmetrix_gb300.build import build
    from symmetrix_gb300.lammps import MODES, PairAdapter
    from symmetrix_gb300.synth.structures import lammps_rank, random_box

    build()
    path = engine_model_path(model_path())
    W = WORKLOAD
    pos, L, species = random_box(W["n_atoms"], W["density"], W["min_dist"], W["n_species"], seed=W["struct_seed"])
    n = len(pos)
    rc = W["r_cut"]
    t = time.time()
    x, local_of, lists = lammps_rank(pos, L, rc + 1.0, 2 * rc + 1.0)
    nall = len(x)
    log(f"LAMMPS layout: {n} local + {nall - n} ghost atoms, {sum(len(a) for a in lists)} list entries "
        f"({time.time() - t:.1f} s)")
    types = (species[local_of] + 1).astype(np.int32)
    mace_types = np.arange(W["n_species"], dtype=np.int32)

    def fold(f):
        out = np.zeros((n, 3))
        np.add.at(out, local_of, f)
        return out

    out = {}
    for form in ("fp32", "bf16"):
        eng = MACE(path, precision=form)
        base = None
        for mode in MODES:
            pair = PairAdapter(eng, mace_types, mode)
            halo = mode == "no_mpi_message_passing"
            call = (lambda changed: pair.compute(x, types, None, np.arange(nall), lists, neigh_changed=changed,
                                                 gnum=nall - n)) if halo else \
                   (lambda changed: pair.compute(x, types, local_of, np.arange(n), lists[:n], neigh_changed=changed))
            res = call(True)
            for _ in range(args.warmup - 1):
                res = call(False)
            times = []
            for _ in range(args.steps):
                t0 = time.perf_counter()
                res = call(False)
                times.append(time.perf_counter() - t0)
            T = float(np.median(times))
            e, f, _, vir = res
            r = {"value": n / T, "ms_per_call": T * 1e3, "ms_mean": float(np.mean(times)) * 1e3}
            if base is None:
                base = (e, fold(f), vir)
            else:
                r["vs_first_mode"] = {"energy_eV": sig(abs(e - base[0]), 3),
                                      "max_folded_force_eV_per_A": sig(float(np.abs(fold(f) - base[1]).max()), 3),
                                      "max_virial_eV": sig(float(np.abs(vir - base[2]).max()), 3)}
            out.setdefault(mode, {})[form] = r
            log(f"{form} {mode}: {r}")
            del pair
        del eng
    first = next(iter(MODES))
    print(json.dumps({
        "metric": "atom-steps/s (one pair_style symmetrix/mace compute() per step, host arrays in and out)",
        "value": out[first]["bf16"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": out[first]["bf16"]["ms_per_call"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": f"pair_modes_4096: the headline box and model as one LAMMPS rank, {n} local and "
                               f"{nall - n} ghost atoms ({2 * rc + 1.0:g} A shell), full lists within "
                               f"{rc + 1.0:g} A of every atom; median host time of one compute() per mode",
                   "atoms": n, "ghosts": nall - n},
        "h2d_bytes_per_call": 8 * 3 * nall, "d2h_bytes_per_call": 8 * 3 * nall,
        "modes": out,
    }), flush=True)


def large_arm(args):
    """MD of the 1,048,576-atom box in both forms (one engine alive at a time: the node
    features of one form take ~90 GB)."""
    import gc

    import torch

    from symmetrix_gb300 import MACE
    from symmetrix_gb300.build import build
    from symmetrix_gb300.md import MD
    from symmetrix_gb300.synth.structures import maxwell_boltzmann, random_box, species_masses

    build()
    json_path = model_path()
    path = engine_model_path(json_path)
    W = WORKLOAD
    sfile = os.path.join(CACHE, f"{W['name']}_s{W['struct_seed']}.npz")
    if os.path.exists(sfile):
        z = np.load(sfile)
        pos, L, species = z["pos"], float(z["L"]), z["species"]
    else:
        t = time.time()
        pos, L, species = random_box(W["n_atoms"], W["density"], W["min_dist"], W["n_species"], seed=W["struct_seed"])
        np.savez(sfile, pos=pos, L=L, species=species)
        log(f"structure built in {time.time() - t:.0f} s")
    N = len(pos)
    dev = torch.device("cuda", 0)
    out = {}
    # errors on a 4096-atom box of the same model, density and species mix
    _, _, sp_e, nl_e = structure(W["err_atoms"], W["struct_seed"] + 100)
    a_e = edge_tuple(sp_e, nl_e)
    ref, _ = oracle_eval(json_path, a_e, host_threads())
    for form in ("fp32", "bf16"):
        eng = MACE(path, precision=form)
        estream = torch.cuda.ExternalStream(eng.stream, device=dev)
        masses = species_masses(eng.atomic_numbers, species)
        vel = maxwell_boltzmann(masses, 300.0, np.random.default_rng(3))
        md = MD(eng, pos, species, masses, box=L, velocities=vel, dt=0.5, skin=1.0, rebuild_every=10)
        md.run(args.warmup)
        md.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(estream)
        md.run(args.steps)
        e1.record(estream)
        md.sync()
        T = e0.elapsed_time(e1) / 1e3
        st = md.state()
        out[form] = {"value": N * args.steps / T, "ms_per_step": T / args.steps * 1e3, "edges_skin_list": md.num_edges,
                     "potential_energy_per_atom": st["potential_energy"] / N}
        del md
        eng.compute_node_energies_forces(*a_e)
        out[form]["errors_vs_fp64"] = dict(box=f"a {W['err_atoms']}-atom box of the same model, density and species "
                                               f"mix ({len(nl_e['r'])} edges)",
                                           **errors(eng.node_energies, eng.node_forces, ref, nl_e))
        del eng
        gc.collect()
    print(json.dumps({
        "metric": METRIC, "value": out["bf16"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": out["bf16"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": W["text"] + "; MD dt 0.5 fs, neighbour list rebuilt every 10 steps (1 A skin), CUDA "
                   "graph between rebuilds", "atoms": N},
        "forms": out, "bf16_over_fp32": out["bf16"]["value"] / out["fp32"]["value"],
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--detail", default=None, help="write the long form of the result to this JSON file")
    ap.add_argument("--full-check", action="store_true",
                    help="precision_32768 / large_1m: also check the whole timed box against the float64 oracle")
    ap.add_argument("--workload", default="fp32_4096",
                    choices=["fp32_4096", "precision_32768", "large_1m", "molecules", "pair_modes"],
                    help="fp32_4096: the headline line; precision_32768: L_max 2, 10 species, 32768 atoms; "
                         "molecules: the batching form (2048 molecules); pair_modes: the headline box through "
                         "the LAMMPS pair-style adapter in its three modes")
    args = ap.parse_args()
    global WORKLOAD
    if args.workload in WORKLOADS:
        WORKLOAD = WORKLOADS[args.workload]
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        reference_arm(args, rank, world)
    elif args.workload == "molecules":
        if rank == 0:
            molecules_arm(args)
    elif args.workload == "large_1m":
        if rank == 0:
            large_arm(args)
    elif args.workload == "pair_modes":
        if rank == 0:
            pair_modes_arm(args)
    else:
        gpu_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
