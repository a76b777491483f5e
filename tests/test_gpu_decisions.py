"""Bin indices and window decisions of the kernels that ship, bit for bit.

The FP32 split path must place every trajectory step in the bins the
reference places it in: round((ts - t0)/dt) and the window tests
ts <= tmin, ts < tmax (src/particle.cpp:780-781, 793, 805, 831-833).  The
production kernels -- the pair kernel in its default form (variant 4) and
with the packed multi-bin deposit (variant 8), and the persistent batched
kernel -- are compiled a second time with one more store per point, which
records the decision each point actually received (re-anchored 16-step
chunks, fast-path votes and exact fallbacks included).  The record is
compared with the oracle's decision for every (pixel, particle, point), and
the recording run's traces with the shipping kernel's, which they must equal
bit for bit (the recording changes no arithmetic).
"""
import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import abi, harness as H

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5
IDX_MASK = (1 << 27) - 1
FLAG_SHIFT = 27
CONFLICT = 1 << 30


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def check_record(dev, ref):
    """Every recorded decision equals the reference's (bin index and the two
    window flags); every point of a step the reference deposits was
    recorded.  Returns (decisions compared, exact fallbacks)."""
    assert dev.shape == ref.shape
    assert not np.any(dev & CONFLICT), "a point received two different decisions"
    written = dev != 0
    dev_idx = dev & IDX_MASK
    ref_idx = ref & IDX_MASK
    dev_fl = (dev >> FLAG_SHIFT) & 3
    ref_fl = (ref >> FLAG_SHIFT) & 3
    bad = written & ((dev_idx != ref_idx) | (dev_fl != ref_fl))
    assert not np.any(bad), f"{int(bad.sum())} decisions differ from the reference's, first at " \
                            f"{np.argwhere(bad)[:5].tolist()}"
    # steps the reference deposits: ts2 > tmin and ts1 < tmax
    f1 = ref_fl[..., :-1]
    f2 = ref_fl[..., 1:]
    real = (ref[..., :-1] != 0) & (ref[..., 1:] != 0)
    dep = real & ((f2 & 1) == 0) & ((f1 & 2) != 0)
    missing = dep & ~(written[..., :-1] & written[..., 1:])
    assert not np.any(missing), f"{int(missing.sum())} in-window steps without a decision"
    fallbacks = int(np.count_nonzero((dev >> (FLAG_SHIFT + 2)) & 1))
    return int(written.sum()), int(dep.sum()), fallbacks


def edge_and_random_pixels(w, n, seed):
    """Pixels of a square screen: its four corners, the middles of its edges
    and its centre, plus a seeded random sample."""
    side = int(round(np.sqrt(w.n_pix)))
    c, e = side // 2, side - 1
    fixed = [0, e, e * side, e * side + e, c, c * side, c * side + e, e * side + c,
             c * side + c]
    rng = np.random.default_rng(seed)
    rest = rng.choice(np.setdiff1d(np.arange(w.n_pix), fixed), n - len(fixed), replace=False)
    return np.sort(np.concatenate([fixed, rest]))


def central_pixels(w, n):
    side = int(round(np.sqrt(w.n_pix)))
    c = side // 2
    d = np.hypot(*np.meshgrid(np.arange(side) - c, np.arange(side) - c, indexing="ij")).ravel()
    return np.sort(np.argsort(d, kind="stable")[:n])


@pytest.fixture(scope="module")
def c4_64():
    w = H.config4(count=64)
    return w.pixel_subset(edge_and_random_pixels(w, 256, 4))


@pytest.mark.parametrize("variant", [4, 8])
def test_config4_shipping_kernel_decisions(c4_64, variant):
    w = c4_64
    ref = lw.screen_decisions(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
    with abi.TrajSet(w.traj) as ts:
        tr_rec, rec = ts.record_decisions(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=variant)
        tr = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=variant)
    n, n_dep, fb = check_record(rec, ref)
    assert n >= 1_000_000 and n_dep > 0
    assert np.array_equal(tr_rec, tr), "the recording instantiation changed the traces"
    oracle, rc = lw.integrate_screen(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
    assert rc == 0
    assert rel_l2(tr, oracle) < TOL_FP32


@pytest.mark.parametrize("variant", [4, 8, 9])
def test_config5_shipping_kernel_decisions(variant):
    """gamma = 2000, 1 as bins: steps span several bins, chains re-anchor
    every chunk and exact fallbacks are frequent."""
    w = H.config5(count=24)
    w = w.pixel_subset(central_pixels(w, 96))
    ref = lw.screen_decisions(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
    with abi.TrajSet(w.traj) as ts:
        tr_rec, rec = ts.record_decisions(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=variant)
        tr = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=variant)
    n, n_dep, fb = check_record(rec, ref)
    # the chained kernels fall back to the exact evaluation near bin edges;
    # the FP64-time kernel (9) evaluates every point so
    assert n >= 1_000_000 and n_dep > 0 and fb > 0
    assert np.array_equal(tr_rec, tr)


def test_config4_decisions_across_slots(c4_64):
    """Many slots: slot boundaries fall inside particles' trajectories, whose
    boundary points are then decided by two blocks."""
    w = c4_64
    ref = lw.screen_decisions(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
    with abi.TrajSet(w.traj) as ts:
        tr_rec, rec = ts.record_decisions(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=4,
                                          n_slots=40)
        tr = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=4, n_slots=40)
    check_record(rec, ref)
    assert np.array_equal(tr_rec, tr)


def test_batched_kernel_decisions():
    """The persistent batched kernel on two uneven config-3 screens: the
    record of one observer against the oracle, and the recorded run's traces
    equal to a replay of the batch's graph."""
    import torch
    dev = torch.device("cuda", 0)
    specs = H.config3_specs()
    order = np.argsort([s["npix"] for s in specs])
    ws = [H.config3_screen(specs[order[0]], count=40), H.config3_screen(specs[order[1]], count=24)]
    sets, bufs, obs = [], [], []
    for w in ws:
        ts = abi.TrajSet(w.traj)
        pos = torch.from_numpy(np.ascontiguousarray(w.pix_pos)).to(dev)
        t0 = torch.from_numpy(np.ascontiguousarray(w.pix_t0)).to(dev)
        out = torch.zeros((w.n_pix, w.nots, 6), dtype=torch.float64, device=dev)
        sets.append(ts)
        bufs.append((pos, t0, out))
        obs.append((ts, pos.data_ptr(), t0.data_ptr(), w.dt, w.nots, w.n_pix, out.data_ptr()))
    try:
        with abi.Batch(obs) as b:
            b.run()
            st, _, _, _ = b.status()
            assert st == abi.TEUFEL_OK
            replay = [o[2].cpu().numpy().copy() for o in bufs]
            for o in bufs:
                o[2].zero_()
            torch.cuda.synchronize(dev)
            for k in range(2):
                for o in bufs:
                    o[2].zero_()
                torch.cuda.synchronize(dev)
                rec = b.record_decisions(k, ws[k].n_pix, sets[k])
                ref = lw.screen_decisions(ws[k].traj, ws[k].pix_pos, ws[k].pix_t0, ws[k].dt,
                                          ws[k].nots)
                n, n_dep, _ = check_record(rec, ref)
                assert n > 0 and n_dep > 0
                recorded = [o[2].cpu().numpy() for o in bufs]
                for a, r in zip(recorded, replay):
                    assert np.array_equal(a, r), "the recording batch run changed the traces"
    finally:
        for ts in sets:
            ts.free()


def test_config4_full_slot_accuracy():
    """One slot accumulating the full 2048 particles (the FP32 accumulation
    bound of a slot), where the FP32 sums' rounding is largest: the traces
    against the oracle within the FP32-split tolerance."""
    w = H.config4(count=2048)
    w = w.pixel_subset(edge_and_random_pixels(w, 48, 7))
    with abi.TrajSet(w.traj) as ts:
        g = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=4, n_slots=1)
        g8 = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=8, n_slots=1)
    ref, rc = lw.integrate_screen(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
    assert rc == 0
    assert rel_l2(g, ref) < TOL_FP32
    assert rel_l2(g8, ref) < TOL_FP32
