"""Benchmark of the batched MD-DPD step: atom-steps/s on one GB300 (or N GPUs, one replica set each).

Workload: 256 independent brush channels drawn from the seed (grafting density U[0.05,0.3],
chain length U{10..100}, channel width U[10,40], box U[15,40], solvent to 0.8, WCA + FENE + DPD
gamma=5, kT=1, dt=0.005), ~4.7M particles, batched in one context, mixed precision (FP32 pair and
bond arithmetic on fixed-point positions, FP64 integration), graph-captured 10-step chunks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision mixed|fp64]
  python bench.py --workload charged-brush|melt-brush|two-liquid [--steps K] [--warmup W] [--precision mixed|fp64]

A step is one full MD step of all replicas.  `value` times K steps with the state resident on the
device (CUDA events on the library's stream).  `e2e` times the same steps through the C ABI with
the state owned by pinned host buffers: every 10-step chunk uploads r, v, a from the host
(mfa_set_state, which also re-sorts), runs the chunk and reads r, v, a and the energies back.
The working set (~1.5 GB) is far larger than the 129 MB L2, so no flush is needed between steps.
`--impl reference` times the restated reference CPU path (the C/OpenMP oracle: linked cells,
schedule(static,10), per-thread force arrays) on the host cores on a bounded sample of replicas.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s on 1 GB300: batched FP32-force vs plain FP64 (force rel err<=1e-5)"
UNIT = "atom-steps/s"
CHUNK = 10
# steps per mfa_step call of the timed loop of the batched replicas: one graph of 100 steps, with
# the energy record every 10 steps kept on the device (the fort.60/61 series ring); the e2e leg
# keeps 10-step calls with a host round trip of the state after each
STEP_CALL = 100
# algorithmic bytes per particle of the pair kernel: mixed -- int4 fixed-point position and float4
# velocity in, float4 force out; fp64 -- double4 position and velocity in, three doubles out (the
# neighbour list itself, 4 B per entry, is not counted)
PAIR_BYTES = {"mixed": 16 + 16 + 16, "fp64": 32 + 32 + 24}
# the mixed pair kernel with the step's integration in its tail: position and velocity views in
# (16 + 16), info and tag (4 + 4), the FP64 position and velocity in and out (48 + 48), the
# rebuild reference position (16), the next step's views out (16 + 16)
PAIR_INTEG_BYTES = 16 + 16 + 4 + 4 + 48 + 48 + 16 + 16 + 16


def profiled_traffic(precision, n_atoms, skin, separate=False):
    """DRAM bytes of one pair-kernel launch, scaled to n_atoms from the committed ncu summary
    (profiles/k_pair_<precision>_brush_replicas.md): the `traffic_bytes_per_particle_skin_S:`
    line of the profiled skin nearest to `skin` (`traffic_separate_bytes_per_particle_skin_S:` for
    the kernel without the integration), else `traffic_bytes_per_particle:`.
    Returns (bytes, the skin of the profile or None)."""
    per_skin, default = {}, None
    key = "traffic_separate_bytes_per_particle_skin_" if separate else "traffic_bytes_per_particle_skin_"
    try:
        with open(os.path.join(ROOT, "profiles", "k_pair_%s_brush_replicas.md" % precision)) as f:
            for ln in f:
                if ln.startswith(key):
                    k, val = ln.split(":")
                    per_skin[float(k.rsplit("_", 1)[1])] = float(val)
                elif ln.startswith("traffic_bytes_per_particle:"):
                    default = float(ln.split(":")[1])
    except OSError:
        return None, None
    if per_skin:
        sk = min(per_skin, key=lambda x: abs(x - skin))
        return per_skin[sk] * n_atoms, sk
    return (default * n_atoms if default is not None else None), None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if "Active" in v and "Not" not in v})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def make_workload(seed, n_rep):
    from mfa_brush_gb300 import configs
    reps = configs.replicas(n_rep, seed)
    return configs.wca_params(gamma=5.0, kT=1.0, dt=0.005), reps


def oracle_params(**kw):
    """The derived tables of the WCA brush model from the oracle's own restatement of
    init_params.f90 (the CPU legs use no part of the library)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from mfa_brush_gb300 import configs
    oracle.build()
    return oracle.derive_params(configs.wca_inputs(**kw))[0]


def cpu_sample(reps, p, steps, warmup, threads):
    """Restated reference CPU path on the given replicas: (atom-steps/s, atom-steps, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    tot_n, tot_t = 0, 0.0
    for (s, a_type, r0, v) in reps:
        o = oracle.Oracle(p, s, a_type, r0, v)
        if warmup:
            o.step(warmup, threads, 0)
        t0 = time.perf_counter()
        o.step(steps, threads, 0)
        tot_t += time.perf_counter() - t0
        tot_n += s.n_part * steps
        o.close()
    return tot_n / tot_t, tot_n, tot_t


def config1_cpu(steps_all, steps_one):
    """The plain FP64 reference-scale channel (20 x 20 x 20, explicit wall beads on a 1 sigma
    lattice, 40 chains of 30 beads per wall, solvent to 0.8, DPD with its own 1 sigma cut-off) on
    the restated reference CPU path: all host cores and one thread."""
    from mfa_brush_gb300 import configs
    p = oracle_params(gamma=5.0, kT=1.0, dt=0.005, wall=1, dpd_cut_off=1.0)
    rep = configs.explicit_wall_channel(seed=1)
    threads = os.cpu_count() or 1
    va, _, _ = cpu_sample([rep], p, steps_all, 10, threads)
    v1, _, _ = cpu_sample([rep], p, steps_one, 5, 1)
    return {"workload": "20x20x20 channel, explicit wall beads, 40 chains of 30 per wall, solvent to 0.8 "
                        "(%d particles, %d mobile), WCA + FENE + DPD (own 1 sigma cut-off), FP64"
                        % (rep[0].n_part, rep[0].n_mon_tot),
            "all_cores": {"value": va, "unit": UNIT, "cores": threads, "steps": steps_all},
            "one_thread": {"value": v1, "unit": UNIT, "cores": 1, "steps": steps_one},
            "kind": "port"}


def plain_fp64(reps, p, skin, device, every=16, steps=100, warmup=20, call=CHUNK):
    """The plain FP64 step on replicas run one at a time (every `every`-th replica of the set):
    atom-steps/s over the sample, each replica timed with CUDA events on its own stream, in
    mfa_step calls of `call` steps."""
    from mfa_brush_gb300 import md
    tot_n, tot_t, picked = 0, 0.0, 0
    warmup = max(call, warmup)
    for (s, a_type, r0, v) in reps[::every]:
        g = md.MdSystem(p, s, a_type, r0, v, precision="fp64", device=device, skin=skin)
        for _ in range(warmup // call):
            g.step(call)
        g.synchronize()
        g.event_record(0)
        for _ in range(steps // call):
            g.step(call)
        g.event_record(1)
        tot_t += g.event_elapsed(0, 1) / 1000.0
        tot_n += s.n_part * steps
        picked += 1
        g.close()
    return tot_n / tot_t, picked, tot_n // steps


def run_reference(args, rank, world):
    """The restated reference CPU path (the oracle's OpenMP loop, all host threads) on this arm's
    workload: every replica of the set, each advanced `steps` timed steps after `warmup`
    untimed ones (at most 20 and 3, so the run stays within a few minutes), with tables derived
    by the oracle itself."""
    if rank != 0:
        return 0
    from mfa_brush_gb300 import configs
    threads = os.cpu_count() or 1
    p = oracle_params(gamma=5.0, kT=1.0, dt=0.005)
    reps = configs.replicas(args.replicas, args.seed)
    steps, warm = min(args.steps, 20), min(args.warmup, 3)
    v, an, t = cpu_sample(reps, p, steps, warm, threads)
    n = int(sum(r[0].n_part for r in reps))
    desc = "all %d replicas (%d particles), %d timed steps each after %d warm-up, one replica at a time" % (
        len(reps), n, steps, warm)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": 1000 * t / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded brush channels)",
            "config": {"workload": "256 uneven brush-channel replicas, WCA+FENE+DPD", "replicas": len(reps),
                       "particles": n, "timed_steps": steps, "seed": args.seed, "precision": "fp64",
                       "l2_flush": "inputs larger than L2"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


SINGLE = {
    "charged-brush": "charged brush channel 40x40x30, N=40, grafting 0.1, -4 per chain + 1280 +1 "
                     "counterions, slab Ewald (alpha_c 0.81, 8070 k-vectors, r_c 3) + DPD",
    "melt-brush": "melt in brush 100x100x40, grafting 0.2 per wall, N=50, melt N=20 to 0.85, cosine "
                  "bending k_b=2, LJ 2*2^(1/6) with eps_bm=1.2, brush WCA, DPD",
    "two-liquid": "two-liquid Poiseuille channel 200x200x50, grafting 0.15, N=30, liquids A/B layered "
                  "to 0.8, eps_AB=0.5, LJ 2*2^(1/6), f_x=0.01, DPD, z-profiles every step",
}


def run_single(args):
    """One large system (the charged-brush channel or the melt-in-brush channel): the same step,
    timed the same way, with the FP32 roofline of its dominant kernel family: the k-space sums
    (8 FLOP per (k, charged particle) for the structure factor, 15 for the force) or the pair
    kernel (LJ 18 + DPD 22 FLOP per evaluation of an interacting pair, each pair evaluated from
    both sides), against the FP32 FMA throughput measured by mfa_fp32_fma_peak."""
    from mfa_brush_gb300 import abi, build, configs, md
    build.build()
    if args.workload == "charged-brush":
        p, (s, a_type, r0, v) = configs.charged_brush()
    elif args.workload == "melt-brush":
        p, (s, a_type, r0, v) = configs.melt_brush()
    else:
        p, (s, a_type, r0, v) = configs.two_liquid_large()
    skin = 0.5 if args.skin == "auto" else float(args.skin)
    prof = {"profile_from_step": 0} if args.workload == "two-liquid" else {}
    g = md.MdSystem(p, s, a_type, r0, v, precision=args.precision, skin=skin,
                    separate_integrator=args.separate_integrator, **prof)
    done = 0
    while done < args.warmup:
        g.step(CHUNK)
        done += CHUNK
    g.synchronize()
    clk = ClockSampler(0)
    clk.start()
    l0 = g.launch_count()
    rb0 = g.rebuild_count()
    g.event_record(0)
    for _ in range(args.steps // CHUNK):
        g.step(CHUNK)
    g.event_record(1)
    ms = g.event_elapsed(0, 1)
    g.synchronize()
    clocks = clk.stop()
    launches = g.launch_count() - l0
    rebuilds = g.rebuild_count() - rb0
    kt = g.kernel_times(args.kernel_steps)
    t = ms / 1000.0
    n = int(s.n_part)
    peak = abi.f64(0.0)
    roof = None
    if abi.load_library().mfa_fp32_fma_peak(0, abi.C.byref(peak)) == 0:
        if args.workload == "charged-brush":
            nk, nq = g.kspace_info()
            fam, flop = "kspace", 23.0 * nk * nq
            what = "k-space family (k_ks_*), %d k-vectors x %d charged particles" % (nk, nq)
        elif args.workload == "melt-brush":
            npair = len(g.pair_list(0))
            fam, flop = "pair", 2.0 * 40.0 * npair
            what = "k_pair, %d interacting pairs (each evaluated from both sides)" % npair
        else:
            fam, flop, what = None, 0.0, ""
        if fam is None and kt.get("pair", (0, 0))[1]:
            # as for the batched replicas: the algorithmic bytes of the timed pair launches (with
            # the integration in the tail on every kernel_times step but the last) against the
            # measured copy bandwidth
            hbm, peak_kind = peaks()
            fused = args.precision == "mixed" and not args.separate_integrator
            n_fused = args.kernel_steps - 1 if fused else 0
            pb = (n_fused * PAIR_INTEG_BYTES + (args.kernel_steps - n_fused) * PAIR_BYTES[args.precision]) \
                / args.kernel_steps
            achieved = pb * n / (kt["pair"][0] / 1000.0) / 1e9
            roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                    "traffic": None, "peak_kind": peak_kind,
                    "kernel": "k_pair (%s%s): %.0f B per particle per launch, averaged over the %d timed launches"
                              % (args.precision, ", integration fused" if fused else "", pb, args.kernel_steps)}
        elif fam and kt.get(fam, (0, 0))[1]:
            achieved = flop / (kt[fam][0] / 1000.0) / 1e12
            roof = {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                    "frac": achieved / peak.value, "traffic": None, "kernel": what,
                    "peak_kind": "measured (mfa_fp32_fma_peak: FMA chains, 8 warps per sub-partition)"}
    line = {"metric": METRIC, "value": n * args.steps / t, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded %s channel)" % args.workload,
            "config": {"workload": SINGLE[args.workload], "particles": n, "precision": args.precision,
                       "chunk_steps": CHUNK, "skin": skin,
                       "l2_flush": ("inputs larger than L2" if n * 96 > 129e6
                                    else "none: the working set fits in L2")},
            "gpu_launches": int(launches + 11 * rebuilds),
            "rebuilds_per_100_steps": 100.0 * rebuilds / args.steps,
            "kernel_ms": {k: round(v_[0], 5) for k, v_ in kt.items() if v_[1]},
            "roofline": roof,
            "clocks": clocks}
    if args.precision == "mixed" and not args.no_fp64:
        # the same system in the plain FP64 mode (the configuration's reference point)
        g.close()
        gd = md.MdSystem(p, s, a_type, r0, v, precision="fp64", skin=skin)
        for _ in range(2):
            gd.step(CHUNK)
        gd.synchronize()
        gd.event_record(0)
        for _ in range(5):
            gd.step(CHUNK)
        gd.event_record(1)
        fv = n * 5 * CHUNK / (gd.event_elapsed(0, 1) / 1000.0)
        gd.close()
        line["plain_fp64"] = {"value": fv, "unit": UNIT, "steps": 5 * CHUNK,
                              "speedup_of_value": line["value"] / fv}
        print(json.dumps(line), flush=True)
        return 0
    print(json.dumps(line), flush=True)
    g.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="brush-replicas",
                    choices=["brush-replicas", "charged-brush", "melt-brush", "two-liquid"],
                    help="brush-replicas: the benchmark; charged-brush: the slab-Ewald channel; "
                         "melt-brush: the 340k-particle melt-in-brush channel; two-liquid: the "
                         "1.6M-particle two-liquid Poiseuille channel with z-profiles")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=60)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--replicas", type=int, default=256)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--kernel-steps", type=int, default=20)
    ap.add_argument("--block", type=int, default=128,
                    help="threads per block of the pair kernel (32, 64, 128); tuned with --skin auto")
    ap.add_argument("--list-cells", type=int, default=0,
                    help="list-build cells per list cut-off (1, 2, 3; 0 = the library's choice)")
    ap.add_argument("--list-cells-x", type=int, default=0,
                    help="list-build cells per list cut-off along x alone (0 = as --list-cells)")
    ap.add_argument("--separate-integrator", action="store_true",
                    help="a separate integrator kernel on every step (default: fused into the pair kernel)")
    ap.add_argument("--pair-schedule", type=int, default=0,
                    help="pair kernel schedule: 0 one block per tile, 1 persistent blocks over a tile queue")
    ap.add_argument("--skin", default="auto",
                    help="list skin in sigma, or 'auto': the whole set timed at 0.3-0.8, then the list cell size, the pair block size and schedule at the chosen skin")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    args.steps = max(CHUNK, (args.steps // CHUNK) * CHUNK)
    # the batched replicas run calls of STEP_CALL steps when the timed steps are a multiple of it,
    # else calls of CHUNK; the warm-up is a whole number of calls (and captures the call's graph)
    args.call = STEP_CALL if args.steps % STEP_CALL == 0 else CHUNK
    args.warmup = -(-args.warmup // args.call) * args.call

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.workload in SINGLE:
        if args.impl == "reference" or world > 1:
            print(json.dumps({"impl": args.impl, "unavailable": "the %s workload is timed for the "
                              "library on one GPU only" % args.workload}), flush=True)
            return 0
        return run_single(args)
    if args.impl == "reference":
        r = run_reference(args, rank, world)
        if dist is not None:
            dist.destroy_process_group()
        return r

    from mfa_brush_gb300 import build, md, shard
    build.build()
    # weak scaling: a global set of replicas x world replicas, split by atom count; rank r
    # generates and runs only its share (the whole set when world == 1)
    from mfa_brush_gb300 import configs
    p = configs.wca_params(gamma=5.0, kT=1.0, dt=0.005)
    rep_idx, reps = shard.rank_replicas(args.replicas, args.seed, rank, world)
    systems, a_type, r0, v = configs.concat(reps)
    n_atoms = int(sum(s.n_part for s in systems))
    tuned = None
    if args.skin == "auto":
        from mfa_brush_gb300 import tune
        # every replica of this rank: the rebuild rate depends on the size of the batch
        # each candidate warmed up like the timed run (the first steps after the lattice start
        # are hotter and rebuild more often)
        best, rates = tune.tune_skin(p, reps, candidates=(0.3, 0.4, 0.5, 0.6, 0.7, 0.8), n_sample=len(reps),
                                     steps=100, warmup=args.warmup, precision=args.precision, device=local,
                                     chunk=100, list_cells=args.list_cells)
        kw = dict(n_sample=len(reps), steps=100, warmup=args.warmup, precision=args.precision, device=local,
                  chunk=100)
        lc, lrates = tune.tune_option(p, reps, best, "list_cells", (1, 2, 3), **kw)
        blk, brates = tune.tune_block(p, reps, best, list_cells=lc, **kw)
        sch, srates = tune.tune_option(p, reps, best, "pair_schedule", (0, 1), list_cells=lc, block_size=blk, **kw)
        tuned = {"candidates": {str(k): round(v_ / 1e9, 4) for k, v_ in rates.items()},
                 "list_cells_candidates": {str(k): round(v_ / 1e9, 4) for k, v_ in lrates.items()},
                 "block_candidates": {str(k): round(v_ / 1e9, 4) for k, v_ in brates.items()},
                 "pair_schedule_candidates": {str(k): round(v_ / 1e9, 4) for k, v_ in srates.items()},
                 "block_size": blk, "list_cells": lc, "pair_schedule": sch,
                 "unit": "G atom-steps/s on the %d replicas of this GPU, 100 steps each after %d "
                         "warm-up steps" % (len(reps), args.warmup)}
        args.skin = best
        args.block = blk
        args.list_cells = lc
        args.pair_schedule = sch
    args.skin = float(args.skin)
    g = md.MdSystem(p, systems, a_type, r0, v, precision=args.precision, device=local, skin=args.skin,
                    block_size=args.block, list_cells=args.list_cells, pair_schedule=args.pair_schedule,
                    separate_integrator=args.separate_integrator, series_capacity=2 * STEP_CALL // CHUNK,
                    list_cells_x=args.list_cells_x)

    def barrier():
        if dist is not None:
            dist.barrier()

    # warm-up (also captures the step graph)
    done = 0
    while done < args.warmup:
        g.step(args.call)
        done += args.call
    g.synchronize()
    barrier()
    clk = ClockSampler(local)
    clk.start()
    rb0 = g.rebuild_count()
    rr0 = g.replica_rebuild_counts()
    l0 = g.launch_count()
    g.synchronize()
    g.event_record(0)
    for _ in range(args.steps // args.call):
        g.step(args.call)
    g.event_record(1)
    ms = g.event_elapsed(0, 1)
    g.synchronize()
    clocks = clk.stop()
    launches = g.launch_count() - l0
    rebuilds = g.rebuild_count() - rb0
    rep_rb = (g.replica_rebuild_counts() - rr0) * (100.0 / args.steps)
    n_rep_part = np.array([s.n_part for s in systems], np.float64)
    t = ms / 1000.0
    # the slowest rank's time; the atom count and per-replica energies of every rank (the one
    # end-of-run gather: E/N of each replica of the global set, in global order, on rank 0)
    dev = "cuda:%d" % local
    t = shard.max_over_ranks(t, dist, dev)
    e_rows = [[e["e_total"] * e["inv_n"], float(s.n_part)] for e, s in zip(g.energies(), systems)]
    e_all = shard.gather_per_replica(e_rows, rep_idx, args.replicas * world, dist)
    n_all = int(e_all[:, 1].sum()) if e_all is not None else n_atoms * world
    value = n_all * args.steps / t

    # per-kernel device times (un-graphed, events around each kernel family)
    kt = g.kernel_times(args.kernel_steps)
    hbm, peak_kind = peaks()
    t_pair = kt["pair"][0] / 1000.0
    # kernel_times runs its steps as mfa_step does: with the integration fused, every step but the
    # last (the energy step) runs the pair kernel with the integration in its tail
    fused = args.precision == "mixed" and not args.separate_integrator and args.pair_schedule == 0
    n_fused = args.kernel_steps - 1 if fused else 0
    pair_bytes = (n_fused * PAIR_INTEG_BYTES + (args.kernel_steps - n_fused) * PAIR_BYTES[args.precision]) \
        / args.kernel_steps
    achieved = pair_bytes * n_atoms / t_pair / 1e9 if t_pair > 0 else 0.0
    traffic, traffic_skin = profiled_traffic(args.precision, n_atoms, args.skin,
                                             separate=args.precision == "mixed" and not fused)

    # end-to-end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(g, n_atoms, n_all, args, dist)

    if e_all is not None and not np.all(np.isfinite(e_all[:, 0])):
        raise RuntimeError("non-finite replica energy after the timed steps")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded brush channels)",
            "config": {"workload": "256 uneven brush-channel replicas, WCA+FENE+DPD, batched",
                       "replicas": args.replicas * world, "particles_per_gpu": n_atoms,
                       "particles_total": n_all, "seed": args.seed,
                       "precision": args.precision, "steps_per_call": args.call,
                       "energy_record": "every %d steps on the device, kept in the energy-series ring" % CHUNK,
                       "skin": args.skin,
                       "pair_block": args.block, "list_cells": g.list_cells(),
                       "list_cells_x": g.options_in_use().list_cells_x, "pair_schedule": args.pair_schedule,
                       "integration": "fused into the pair kernel" if fused else "separate kernel",
                       "skin_autotune": tuned,
                       "l2_flush": "inputs larger than L2 (~1.5 GB working set)",
                       "parallelism": "replicas" if world == 1 else "replicas x %d GPUs" % world},
            "gpu_launches": int(launches + 11 * rebuilds),
            "rebuilds_per_100_steps": 100.0 * rebuilds / args.steps,
            "replica_rebuilds_per_100_steps": {
                "mean": float(rep_rb.mean()), "min": float(rep_rb.min()), "max": float(rep_rb.max()),
                "particle_weighted": float((rep_rb * n_rep_part).sum() / n_rep_part.sum()),
                "note": "a replica is rebuilt when its own particles moved half the skin; a step with "
                        "any rebuild counts once in rebuilds_per_100_steps"},
            "kernel_ms": {k: round(v_[0], 5) for k, v_ in kt.items() if v_[1]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic,
                         "kernel": "k_pair (%s%s): %.0f B per particle per launch, averaged over the "
                                   "%d timed launches" % (args.precision, ", integration fused" if fused else "",
                                                          pair_bytes, args.kernel_steps),
                         "traffic_source": "ncu DRAM bytes per particle of one full launch at skin %s "
                                           "(profiles/k_pair_%s_brush_replicas.md), times N"
                                           % (traffic_skin, args.precision),
                         "peak_kind": peak_kind},
            "clocks": clocks}
    if e2e is not None:
        line["e2e"] = e2e
    if rank == 0 and not args.no_fp64:
        # the reference point of the batched mixed step: the same kind of replicas advanced one at
        # a time in plain FP64
        fv, fk, fn = plain_fp64(reps, p, args.skin, local, call=args.call)
        line["plain_fp64_one_at_a_time"] = {
            "value": fv, "unit": UNIT, "replicas": fk, "particles": int(fn), "steps": 100,
            "sample": "every 16th replica of the set, each alone in its own FP64 context, %d-step graphs" % args.call,
            "speedup_of_value": value / world / fv}
        # the same batch in the plain FP64 mode (precision alone, batching held fixed)
        gd = md.MdSystem(p, systems, a_type, r0, v, precision="fp64", device=local, skin=args.skin,
                         list_cells=args.list_cells)
        nb = max(1, 100 // args.call)  # 100 steps in the timed loop's calls
        for _ in range(max(1, 20 // args.call)):
            gd.step(args.call)
        gd.synchronize()
        gd.event_record(0)
        for _ in range(nb):
            gd.step(args.call)
        gd.event_record(1)
        bv = n_atoms * nb * args.call / (gd.event_elapsed(0, 1) / 1000.0)
        gd.close()
        line["batched_fp64"] = {"value": bv, "unit": UNIT, "steps": nb * args.call, "steps_per_call": args.call,
                                "speedup_of_value": value / world / bv}
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sample, n = [], 0
        for r in reps:
            if n > 60000:
                break
            sample.append(r)
            n += r[0].n_part
        po = oracle_params(gamma=5.0, kT=1.0, dt=0.005)
        cv, an, ct = cpu_sample(sample, po, 40, 5, threads)
        line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d replicas, %d particles, 40 steps (restated reference "
                                          "OpenMP path)" % (len(sample), n)}
        # the same path on one thread, on the first replica only (a few seconds)
        c1, _, _ = cpu_sample(sample[:1], po, 20, 2, 1)
        line["cpu_baseline_1thread"] = {"value": c1, "unit": UNIT, "cores": 1, "kind": "port",
                                        "sample": "1 replica, %d particles, 20 steps" % sample[0][0].n_part}
        line["cpu_baseline_config1"] = config1_cpu(2000, 400)
    if rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_e2e(g, n_atoms, n_all, args, dist):
    import torch
    from mfa_brush_gb300 import abi
    shape = (n_atoms, 3)
    hr = torch.empty(shape, dtype=torch.float64, pin_memory=torch.cuda.is_available()).numpy()
    hv = torch.empty(shape, dtype=torch.float64, pin_memory=torch.cuda.is_available()).numpy()
    ha = torch.empty(shape, dtype=torch.float64, pin_memory=torch.cuda.is_available()).numpy()
    lib = abi.load_library()
    dp = abi.dptr
    abi.check(lib.mfa_sync_to_host(g.ctx, dp(hr), dp(hv), dp(ha), None), g.ctx)
    e = (abi.Energies * g.nrep)()
    chunks = max(1, min(args.steps, 300) // CHUNK)
    # one untimed round trip
    abi.check(lib.mfa_set_state(g.ctx, dp(hr), dp(hv), dp(ha)), g.ctx)
    g.step(CHUNK)
    abi.check(lib.mfa_sync_to_host(g.ctx, dp(hr), dp(hv), dp(ha), None), g.ctx)
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(chunks):
        abi.check(lib.mfa_set_state(g.ctx, dp(hr), dp(hv), dp(ha)), g.ctx)  # H2D
        g.step(CHUNK)
        abi.check(lib.mfa_sync_to_host(g.ctx, dp(hr), dp(hv), dp(ha), None), g.ctx)  # D2H
        abi.check(lib.mfa_get_energies(g.ctx, e), g.ctx)
    t = time.perf_counter() - t0
    from mfa_brush_gb300 import shard
    t = shard.max_over_ranks(t, dist, "cuda:%d" % torch.cuda.current_device() if torch.cuda.is_available() else "cpu")
    steps = chunks * CHUNK
    bytes_state = 3 * 3 * 8 * n_atoms
    return {"value": n_all * steps / t, "unit": UNIT,
            "h2d_bytes_per_step": bytes_state // CHUNK,
            "d2h_bytes_per_step": (bytes_state + g.nrep * 104) // CHUNK,
            "steps": steps, "pattern": "per 10-step chunk: r,v,a H2D (mfa_set_state) + mfa_step(10) + "
                                       "r,v,a D2H (mfa_sync_to_host) + energies"}


if __name__ == "__main__":
    sys.exit(main())
