"""Per-frame output from the GPU (needs a GPU): ``write_files(wait=False)``
snapshots the frame on the solver's stream, copies it to pinned host memory on a
side stream and writes its files on a background thread while the run steps on.
Its files must equal, byte for byte, those a synchronous ``write_files()`` of
the same frame writes (main.py:371-378)."""
import filecmp
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sim(out):
    from tichi_sph_gb300 import sph_config, workloads
    from tichi_sph_gb300.simulation import Simulation
    cfg_d, scen_d = workloads.dambreak_2d()
    cfg = sph_config.Config(cfg_d, scen_d)
    sim = Simulation(cfg, device="cuda", out_dir=str(out))
    sim.init_scenario()
    return sim


def test_async_frames_equal_synchronous_frames(tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    a, b = _sim(tmp_path / "async"), _sim(tmp_path / "sync")
    try:
        for frame in range(1, 7):
            for sim in (a, b):
                sim.globalvar.time_counter = frame
                for _ in range(3):
                    sim.substep()
            a.write_files(wait=False)   # returns before the copy ends; the next substeps overwrite pos / vel
            b.write_files()
        a.flush()
    finally:
        a.solver.close()
        b.solver.close()
    for sub in ("ply", "json", "part_data"):
        names = sorted(os.listdir(tmp_path / "sync" / sub))
        assert names == sorted(os.listdir(tmp_path / "async" / sub))
        assert len(names) == (12 if sub == "part_data" else 6)
        for nm in names:
            assert filecmp.cmp(tmp_path / "sync" / sub / nm, tmp_path / "async" / sub / nm, shallow=False), (sub, nm)
    pos = np.load(tmp_path / "async" / "part_data" / "pos_6.npy")
    assert pos.shape == (5000, 2) and np.isfinite(pos).all()
