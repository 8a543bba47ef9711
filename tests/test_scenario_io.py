"""Host side of run-time scenario emission and per-frame output (CPU, no
stepping): inlets and delayed objects (main.py:26-112, sph_obj.py:117-137),
the PLY writer (sph_util.py:90-100) and the files of one frame (main.py:371-378,
the frame JSON of main.py:151-171), written at once or by the background
writer."""
import json
import os

import numpy as np
import pytest

from tichi_sph_gb300 import sph_config, workloads
from tichi_sph_gb300.simulation import Simulation, read_ply, write_ply

PS = 0.02
COLOR = "0x6F7DBC"


def _sim(tmp_path, objs):
    cfg = workloads._config(cs=20)
    scen = {
        "sim_env": {"global_part_size": PS, "global_dynamic_viscosity": 0.01, "sim_dim": 3,
                    "sim_space_lb": [-1.0, -1.0, -1.0], "sim_space_rt": [1.0, 1.0, 1.0],
                    "gravity": [0, -9.81, 0], "phase_num": 1, "phase_rest_density": [1000],
                    "phase_color_hex": [COLOR]},
        "fluid": {"max_part_num": 20000, "objs": objs},
        "bound": {"max_part_num": 10, "objs": []},
    }
    sim = Simulation(sph_config.Config(cfg, scen), device="cpu", out_dir=str(tmp_path / "out"))
    sim.init_scenario()
    return sim


def _cube(start, end, **extra):
    o = workloads._obj("cube", start, end, [1], [0, 0, 0])
    o.update(extra)
    return o


@pytest.mark.parametrize("dim", [2, 3])
def test_ply_round_trip(tmp_path, dim):
    """ASCII PLY with float x, y, z (z = 0 in 2D) of the first num positions;
    the values read back are the FP32 positions exactly."""
    pos = np.random.default_rng(1).uniform(-1, 1, (50, dim)).astype(np.float32)
    write_ply(tmp_path / "fluid_pos", 7, dim, 40, pos)
    path = tmp_path / "fluid_pos_7.ply"
    head = path.read_text().splitlines()[:7]
    assert head == ["ply", "format ascii 1.0", "element vertex 40", "property float x", "property float y",
                    "property float z", "end_header"]
    want = np.zeros((40, 3), np.float32)
    want[:, :dim] = pos[:40]
    np.testing.assert_array_equal(read_ply(str(path)).astype(np.float32), want)


def test_inlet_pushes_on_the_reference_schedule(tmp_path):
    """An inlet pointing down pushes a layer at once and then whenever the
    clock has advanced by dt = (sqrt(v^2 + 2 a r) - v) / a * rf (a = the
    gravity along the inlet normal, r = part_size; main.py:26-39), each layer
    moving at speed along the normal, until its end time."""
    inlet = {"type": "inlet", "center": [0.0, 0.5, 0.0], "size": [0.1, 0.1], "norm": [0, -1, 0], "speed": 1.0,
             "volume_frac": [1], "color": COLOR, "particle_relaxing_factor": 1.0, "end_time": 0.1}
    sim = _sim(tmp_path, [inlet])
    fl, gv = sim.fluid, sim.globalvar
    a, v, r = 9.81, 1.0, float(np.float32(PS))
    dt = (np.sqrt(v * v + 2 * a * r) - v) / a
    assert sim.inlets[0]["dt"] == pytest.approx(dt, rel=1e-6)
    pushes = []
    n_prev = fl.part_num[None]
    for k in range(200):
        gv.time_count = k * 1e-3
        sim.refresh_scenario()
        n = fl.part_num[None]
        if n != n_prev:
            pushes.append((gv.time_count, n - n_prev))
            vel = fl.vel[n_prev:n].numpy()
            np.testing.assert_allclose(vel, np.tile([0.0, -1.0, 0.0], (n - n_prev, 1)), atol=1e-7)
            n_prev = n
    times = [t for t, _ in pushes]
    # the first layer at t = 0; each later one at the first clock tick past t_pre + dt
    want, t_pre = [], None
    for k in range(200):
        t = k * 1e-3
        if t >= 0.1:
            break
        if t_pre is None or t >= t_pre + dt:
            want.append(t)
            t_pre = t
    assert times == pytest.approx(want)
    counts = {c for _, c in pushes}
    assert len(counts) == 1 and counts.pop() == 25  # 5 x 5 layer of 0.1 x 0.1 at spacing 0.02
    assert not sim.inlets  # removed once its end time has passed


def test_delayed_object_appears_at_its_time(tmp_path):
    """An object with a positive time waits in the scenario buffer
    (main.py:66-72) and is emitted by the first refresh at or after that time
    (main.py:102-109)."""
    sim = _sim(tmp_path, [_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1]),
                          _cube([0.3, 0.0, 0.0], [0.4, 0.1, 0.1], time=0.05)])
    fl, gv = sim.fluid, sim.globalvar
    n0 = fl.part_num[None]
    assert n0 == 125 and len(sim.scenario_wait_buffer) == 1
    for t, n_want in ((0.0, n0), (0.049, n0), (0.05, 2 * n0), (0.2, 2 * n0)):
        gv.time_count = t
        sim.refresh_scenario()
        assert fl.part_num[None] == n_want, t
    assert not sim.scenario_wait_buffer
    assert float(fl.pos[n0:2 * n0, 0].min()) > 0.29


def test_frame_files(tmp_path):
    """One frame's files: ply/fluid_pos_<frame>.ply, json/frame<frame>.json with
    the reference's keys, part_data/pos_<frame>.npy and vel_<frame>.npy of the
    fluid's part_num particles."""
    sim = _sim(tmp_path, [_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1], vel=[0.5, 0, 0])])
    sim.globalvar.time_counter = 3
    sim.write_files()
    out = tmp_path / "out"
    n = sim.fluid.part_num[None]
    pos = np.load(out / "part_data" / "pos_3.npy")
    vel = np.load(out / "part_data" / "vel_3.npy")
    assert pos.shape == (n, 3) and vel.shape == (n, 3)
    np.testing.assert_array_equal(pos, sim.fluid.pos[:n].numpy())
    np.testing.assert_array_equal(read_ply(str(out / "ply" / "fluid_pos_3.ply")).astype(np.float32), pos)
    rec = json.loads((out / "json" / "frame3.json").read_text())
    assert set(rec) == {"step", "frame", "timeInSimulation", "timeStep", "fps", "iteration", "energy"}
    assert set(rec["iteration"]) == {"divergenceFree_iteration", "incompressible_iteration", "sum_iteration"}
    assert set(rec["energy"]) == {"statistics_kinetic_energy", "statistics_gravity_potential_energy", "sum_energy"}
    assert rec["frame"] == 3
    assert sorted(os.listdir(out)) == ["json", "part_data", "ply"]


def test_frames_written_in_the_background(tmp_path):
    """write_files(wait=False): each frame's files hold the state at the call,
    although the state changes before the background writes finish; flush waits
    for all of them."""
    import torch
    sim = _sim(tmp_path, [_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1])])
    n = sim.fluid.part_num[None]
    want = {}
    for frame in range(1, 6):
        sim.globalvar.time_counter = frame
        sim.fluid.pos[:n] += torch.tensor([0.01, 0.0, 0.0])
        want[frame] = sim.fluid.pos[:n].numpy().copy()
        sim.write_files(wait=False)
    sim.flush()
    out = tmp_path / "out"
    for frame, pos in want.items():
        np.testing.assert_array_equal(np.load(out / "part_data" / ("pos_%d.npy" % frame)), pos)
        assert json.loads((out / "json" / ("frame%d.json" % frame)).read_text())["frame"] == frame


def test_background_write_error_surfaces_at_flush(tmp_path):
    sim = _sim(tmp_path, [_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1])])
    blocker = tmp_path / "blocked"
    blocker.write_text("a file where the output folder should be")
    sim.out_dir = str(blocker)
    sim.write_files(wait=False)
    with pytest.raises(OSError):
        sim.flush()
    sim.flush()  # the error is reported once


def test_inlet_interval_branches(tmp_path):
    """main.py:26-39 for an inlet whose normal has no downward gravity component
    (dt = r rf / v, or no pushes at all at speed 0) and for a negative speed
    (the normal and the speed both flip)."""
    sim = _sim(tmp_path, [_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1])])
    r = float(np.float32(PS))
    assert sim.inlet_helper_get_dt([0, 1, 0], 2.0, 1.5) == pytest.approx(r * 1.5 / 2.0)
    assert sim.inlet_helper_get_dt([1, 0, 0], 0.5, 1.0) == pytest.approx(r / 0.5)
    assert sim.inlet_helper_get_dt([0, 2, 0], 0.0, 1.0) == float("inf")
    # speed -1 along +y is speed 1 along -y: gravity along the normal, the quadratic branch
    a = 9.81
    assert sim.inlet_helper_get_dt([0, 1, 0], -1.0, 1.0) == pytest.approx((np.sqrt(1 + 2 * a * r) - 1) / a)


def test_frame_writer_queue_is_bounded():
    """A writer slower than the solver holds submit back once max_pending frames
    wait, instead of letting their host copies pile up."""
    import threading
    from tichi_sph_gb300.simulation import FrameWriter
    w = FrameWriter(max_pending=2)
    gate = threading.Event()
    started = threading.Event()

    def slow():
        started.set()
        gate.wait(10)

    w.submit(slow)
    started.wait(10)
    w.submit(lambda: None)
    w.submit(lambda: None)  # the queue now holds its two frames
    t = threading.Thread(target=lambda: w.submit(lambda: None))
    t.start()
    t.join(0.2)
    assert t.is_alive()  # the fourth frame waits for room
    gate.set()
    t.join(10)
    assert not t.is_alive()
    w.flush()
