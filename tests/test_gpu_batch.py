"""Batched uneven observers (teufel_cuda_batch_*): one persistent launch over
a device work queue and one reduction, replayed from a CUDA graph, against
the oracle on a seeded draw of the batched-observer configuration (uneven
meshes, trace lengths, particle counts and trajectory lengths)."""
import numpy as np
import pytest
import torch

from oracle import lw
from teufel_gb300 import abi, harness as H

pytestmark = pytest.mark.gpu
TOL_FP32 = 1e-5


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def screens():
    """Six of the sixteen seeded screens, each with a few particles and an
    evenly spaced pixel subset, so the oracle stays quick."""
    specs = H.config3_specs()
    out = []
    for k in (0, 2, 3, 6, 10, 14):
        w = H.config3_screen(specs[k], count=min(specs[k]["n_particles"], 9 if k else 5))
        step = max(1, w.n_pix // 40)
        out.append(w.pixel_subset(np.arange(0, w.n_pix, step)))
    return out


def test_batch_matches_oracle_and_replays(screens):
    dev = torch.device("cuda:0")
    sets = [abi.TrajSet(w.traj) for w in screens]
    bufs, obs, refs = [], [], []
    for w, ts in zip(screens, sets):
        pos = torch.from_numpy(np.ascontiguousarray(w.pix_pos)).to(dev)
        t0 = torch.from_numpy(np.ascontiguousarray(w.pix_t0)).to(dev)
        out = torch.zeros((w.n_pix, w.nots, 6), dtype=torch.float64, device=dev)
        bufs.append((pos, t0, out))
        obs.append((ts, pos.data_ptr(), t0.data_ptr(), w.dt, w.nots, w.n_pix, out.data_ptr()))
        ref, rc = lw.integrate_screen(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
        assert rc == 0
        refs.append(ref)
    # the first screen again, sharing its trajectory set with a second observer
    w0 = screens[0]
    out_b = torch.zeros((w0.n_pix, w0.nots, 6), dtype=torch.float64, device=dev)
    obs.append((sets[0], bufs[0][0].data_ptr(), bufs[0][1].data_ptr(), w0.dt, w0.nots,
                w0.n_pix, out_b.data_ptr()))
    # an observer without work (one-sample trace) is accepted and skipped
    out_c = torch.ones((3, 1, 6), dtype=torch.float64, device=dev)
    obs.append((sets[1], bufs[1][0].data_ptr(), bufs[1][1].data_ptr(), screens[1].dt, 1, 3,
                out_c.data_ptr()))
    with abi.Batch(obs) as b:
        b.run()
        st, items, inwin, ms = b.status()
        assert st == 0 and items > len(screens) and inwin > 0
        first = [o.cpu().numpy().copy() for _, _, o in bufs]
        for g, ref in zip(first, refs):
            assert rel_l2(g, ref) < TOL_FP32, rel_l2(g, ref)
        assert np.array_equal(out_b.cpu().numpy(), first[0])
        assert torch.all(out_c == 1.0)
        # replaying the graph adds the same result again, bit for bit
        b.run()
        assert b.status()[0] == 0
        for (_, _, o), g in zip(bufs, first):
            assert np.array_equal(o.cpu().numpy(), 2.0 * g)
    for ts in sets:
        ts.free()


def test_batch_rejects_bad_arguments(screens):
    w = screens[1]
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(np.ascontiguousarray(w.pix_pos)).to(dev)
    t0 = torch.from_numpy(np.ascontiguousarray(w.pix_t0)).to(dev)
    out = torch.zeros((w.n_pix, w.nots, 6), dtype=torch.float64, device=dev)
    with abi.TrajSet(w.traj) as ts:
        with pytest.raises(abi.TeufelError):
            abi.Batch([(ts, 0, 0, w.dt, w.nots, w.n_pix, 0)])
        # the batch runs FP32 kernels only: a reversed window (dt < 0) or dt = 0
        for dt in (-w.dt, 0.0):
            with pytest.raises(abi.TeufelError) as ei:
                abi.Batch([(ts, pos.data_ptr(), t0.data_ptr(), dt, w.nots, w.n_pix,
                            out.data_ptr())])
            assert ei.value.status == abi.TEUFEL_ERR_ARG
