"""mfa_pair_list_static (the pair-list export with fixed device scratch) against mfa_pair_list.

Both are called through the C ABI on the same state; the pair sets must be identical (integer
index work: exact), on two calls in a row so that a counter left over from the first call would
show.  Collected last so that it also runs after every other GPU test in one process."""
import ctypes as C

import numpy as np
import pytest

from mfa_brush_gb300 import abi, configs, md

pytestmark = pytest.mark.gpu

STATIC_MAX = 262144  # MFA_PAIR_LIST_STATIC_MAX in include/mfa_gpu.h


def static_pairs(g, rep, cap):
    pairs = np.zeros((max(cap, 1), 2), np.int32)
    n = abi.i64(0)
    rc = g.lib.mfa_pair_list_static(g.ctx, rep, abi.iptr(pairs), cap, C.byref(n))
    return rc, pairs[: min(cap, n.value)], n.value


def as_set(p):
    return set(map(tuple, np.sort(p, axis=1).tolist()))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_pair_list_equals_allocating(gpu, try_deck, precision):
    inp, p, s, a_type, r0, v, a = try_deck
    g = md.MdSystem(p, s, a_type, r0, v, a, precision=precision)
    ref = g.pair_list(0)
    assert len(ref) > 0
    cap = min(STATIC_MAX, 4 * len(ref))
    for _ in range(2):
        rc, got, n = static_pairs(g, 0, cap)
        assert rc == abi.MFA_OK
        assert n == len(ref)
        assert len(got) == n and as_set(got) == as_set(ref)


def test_static_pair_list_after_steps_and_batched(gpu):
    """A batch of two replicas, after a few steps: both replicas, two calls each."""
    p = configs.wca_params(gamma=5.0)
    reps = [configs.brush_channel(15.0, 12.0, 0.2, 20, seed=11),
            configs.brush_channel(18.0, 10.0, 0.15, 15, seed=12)]
    systems, a_type, r0, v = configs.concat(reps)
    g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed")
    g.step(25)
    for rep in range(2):
        ref = g.pair_list(rep)
        for _ in range(2):
            rc, got, n = static_pairs(g, rep, len(ref) + 17)
            assert rc == abi.MFA_OK and n == len(ref)
            assert as_set(got) == as_set(ref)


def test_static_pair_list_limits(gpu, try_deck):
    inp, p, s, a_type, r0, v, a = try_deck
    g = md.MdSystem(p, s, a_type, r0, v, a, precision="fp64")
    ref = g.pair_list(0)
    # a cap below the count stores cap pairs and reports the full count, as mfa_pair_list does
    rc, got, n = static_pairs(g, 0, 10)
    assert rc == abi.MFA_OK and n == len(ref) and len(got) == 10
    assert as_set(got) <= as_set(ref)
    # a cap above the fixed scratch is refused with a message
    rc, _, _ = static_pairs(g, 0, STATIC_MAX + 1)
    assert abi.ERRORS.get(rc) == "MFA_ERR_CAPACITY"
    assert "MFA_PAIR_LIST_STATIC_MAX" in g.lib.mfa_last_error(g.ctx).decode()
    # and the scratch still works afterwards
    rc, got, n = static_pairs(g, 0, STATIC_MAX)
    assert rc == abi.MFA_OK and as_set(got) == as_set(ref)


def test_static_pair_list_takes_no_device_memory(gpu, try_deck):
    """The case the entry point exists for: another component of the host program holds nearly all
    of the device's free memory.  The allocating export then cannot get its scratch and says so
    (MFA_ERR_ALLOC); the static one still returns the same pairs, on two calls in a row, and the
    device's free memory is the same before and after them."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    inp, p, s, a_type, r0, v, a = try_deck
    g = md.MdSystem(p, s, a_type, r0, v, a, precision="mixed")
    ref = g.pair_list(0)
    rc, _, _ = static_pairs(g, 0, len(ref))  # first call on the context: the address lookup
    assert rc == abi.MFA_OK
    free, _ = torch.cuda.mem_get_info(0)
    try:
        hold = torch.empty(free - (192 << 20), dtype=torch.uint8, device="cuda:0")
    except RuntimeError:
        pytest.skip("could not take the device's free memory")
    try:
        pairs = np.zeros((len(ref) + 1, 2), np.int32)
        n = abi.i64(0)
        big = 64 << 20  # 64 Mi pairs: 512 MiB of scratch, more than is left
        rc = g.lib.mfa_pair_list(g.ctx, 0, abi.iptr(pairs), big, C.byref(n))
        assert abi.ERRORS.get(rc) == "MFA_ERR_ALLOC"
        f0, _ = torch.cuda.mem_get_info(0)
        for _ in range(2):
            rc, got, n = static_pairs(g, 0, STATIC_MAX)
            assert rc == abi.MFA_OK and n == len(ref)
            assert as_set(got) == as_set(ref)
        f1, _ = torch.cuda.mem_get_info(0)
        assert f1 == f0
    finally:
        del hold
        torch.cuda.empty_cache()
    # the context goes on working once the memory is back
    g.step(10)
    rc, got, n = static_pairs(g, 0, STATIC_MAX)
    assert rc == abi.MFA_OK and as_set(got) == as_set(g.pair_list(0))
