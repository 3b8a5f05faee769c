"""Autotuning of the neighbour-list skin, the list-build cell size, the pair kernel's block size
and its schedule (one block per tile, or persistent blocks over a tile queue).

The skin trades the list rebuild (sort + list build, whose frequency falls as the skin grows) for
the pair kernel (whose lists lengthen with it).  The best value depends on the density, the
temperature, the time step and the replica mix, so it is measured: the fused step is timed at
each candidate skin, over enough steps to include several rebuilds.  A replica is rebuilt when one
of its own particles has moved half the skin, and a step with any rebuild pays the fixed cost of
the sort's passes over the whole batch, so the rate and cost depend on the batch: time the whole
batch (n_sample >= the replica count) when the tuned skin is for that batch.
"""
import numpy as np

from . import abi, configs, md


def sample_replicas(reps, n_sample):
    """Every k-th replica, so that the sample spans the size distribution of the set."""
    if len(reps) <= n_sample:
        return list(reps)
    idx = np.linspace(0, len(reps) - 1, n_sample).round().astype(int)
    return [reps[k] for k in sorted(set(idx.tolist()))]


def tune_skin(params, reps, candidates=(0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9), n_sample=32, steps=80, warmup=20,
              precision="mixed", device=0, chunk=10, **opt):
    """Times mfa_step on a sample of `reps` (list of (System, a_type, r0, v)) at each candidate
    skin (further keyword arguments are options of every context); returns (best skin,
    {skin: atom-steps/s})."""
    sample = sample_replicas(reps, n_sample)
    systems, a_type, r0, v = configs.concat(sample)
    n_atoms = int(sum(s.n_part for s in systems))
    rates = {}
    for skin in candidates:
        g = md.MdSystem(params, systems, a_type, r0, v, precision=precision, device=device, skin=skin, **opt)
        for _ in range(max(1, warmup // chunk)):
            g.step(chunk)
        g.synchronize()
        g.event_record(0)
        for _ in range(max(1, steps // chunk)):
            g.step(chunk)
        g.event_record(1)
        ms = g.event_elapsed(0, 1)
        g.close()
        rates[float(skin)] = n_atoms * max(1, steps // chunk) * chunk / (ms / 1000.0)
    best = max(rates, key=rates.get)
    return best, rates


def tune_block(params, reps, skin, candidates=(64, 128), n_sample=32, steps=80, warmup=20,
               precision="mixed", device=0, chunk=10, **opt):
    """Times mfa_step at the given skin with each candidate pair-kernel block size (threads per
    block); returns (best block size, {block: atom-steps/s})."""
    sample = sample_replicas(reps, n_sample)
    systems, a_type, r0, v = configs.concat(sample)
    n_atoms = int(sum(s.n_part for s in systems))
    rates = {}
    for b in candidates:
        g = md.MdSystem(params, systems, a_type, r0, v, precision=precision, device=device, skin=skin,
                        block_size=b, **opt)
        for _ in range(max(1, warmup // chunk)):
            g.step(chunk)
        g.synchronize()
        g.event_record(0)
        for _ in range(max(1, steps // chunk)):
            g.step(chunk)
        g.event_record(1)
        ms = g.event_elapsed(0, 1)
        g.close()
        rates[int(b)] = n_atoms * max(1, steps // chunk) * chunk / (ms / 1000.0)
    best = max(rates, key=rates.get)
    return best, rates


def tune_option(params, reps, skin, name, candidates, n_sample=32, steps=80, warmup=20, precision="mixed",
                device=0, chunk=10, **opt):
    """Times mfa_step at the given skin with each candidate value of the context option `name`
    (an mfa_options field: list_cells, pair_schedule, block_size); a candidate that the library
    refuses for these boxes is skipped.  Returns (best value, {value: atom-steps/s})."""
    sample = sample_replicas(reps, n_sample)
    systems, a_type, r0, v = configs.concat(sample)
    n_atoms = int(sum(s.n_part for s in systems))
    rates = {}
    for c in candidates:
        try:
            g = md.MdSystem(params, systems, a_type, r0, v, precision=precision, device=device, skin=skin,
                            **dict(opt, **{name: c}))
        except abi.MfaError:
            continue
        for _ in range(max(1, warmup // chunk)):
            g.step(chunk)
        g.synchronize()
        g.event_record(0)
        for _ in range(max(1, steps // chunk)):
            g.step(chunk)
        g.event_record(1)
        ms = g.event_elapsed(0, 1)
        g.close()
        rates[c] = n_atoms * max(1, steps // chunk) * chunk / (ms / 1000.0)
    best = max(rates, key=rates.get)
    return best, rates
