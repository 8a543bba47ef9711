"""Headless driver: scenario set-up, the time loop and per-frame output.

Mirrors ``main.py`` of Tichi_SPH without its GGUI window (there is no graphics
stack here): the objects of ``main.py:8-14``, the scenario system of
``main.py:16-112`` (cubes, boxes, PLY point clouds, inlets and objects delayed
by ``time``), ``run_step`` (``main.py:339-368``) and the output writers
(``main.py:115-171``, ``371-378``) with portable paths.
"""
import json
import os
import queue
import threading
import time
import warnings

import numpy as np

from .sph import Solver
from .sph_obj import Fluid, GlobalVariable, Grid, Ngrid


def warn(*message):
    """``sph_util.py:77-80``."""
    warnings.warn("".join(str(m) for m in message), RuntimeWarning)


def read_ply(path):
    """ASCII PLY vertex reader (``sph_util.py:83-87`` reads x, y, z of each vertex)."""
    with open(path, "rb") as f:
        header = []
        while True:
            line = f.readline().decode("ascii", errors="replace").strip()
            header.append(line)
            if line == "end_header":
                break
            if not line and len(header) > 200:
                raise ValueError("bad PLY header in %s" % path)
        nvert, props, fmt = 0, [], "ascii"
        in_vertex = False
        for ln in header:
            t = ln.split()
            if not t:
                continue
            if t[0] == "format":
                fmt = t[1]
            elif t[0] == "element":
                in_vertex = t[1] == "vertex"
                if in_vertex:
                    nvert = int(t[2])
            elif t[0] == "property" and in_vertex:
                props.append(t[-1])
        if fmt != "ascii":
            raise ValueError("only ASCII PLY is supported (%s)" % path)
        rows = [f.readline().split() for _ in range(nvert)]
    ix = [props.index(a) for a in ("x", "y", "z")]
    return np.array([[float(r[i]) for i in ix] for r in rows])


def write_ply(path, frame_num, dim, num, pos):
    """``sph_util.py:90-100``: ASCII PLY of the first ``num`` positions."""
    with open(str(path) + "_" + str(frame_num) + ".ply", "w") as f:
        f.write("ply\nformat ascii 1.0\nelement vertex %d\nproperty float x\nproperty float y\n"
                "property float z\nend_header\n" % num)
        for i in range(num):
            z = pos[i, 2] if dim == 3 else 0.0
            f.write("%s %s %s\n" % (np.float32(pos[i, 0]), np.float32(pos[i, 1]), np.float32(z)))


class FrameWriter:
    """Writes frames' files in submission order on one background thread, so
    that the time loop goes on while a frame's PLY / JSON / npy files are
    written.  At most ``max_pending`` frames wait at a time: ``submit`` blocks
    while that many are queued, so a disk slower than the solver holds the time
    loop back instead of piling up host copies.  ``flush`` waits for every
    submitted frame and re-raises the first error a write met."""

    def __init__(self, max_pending=4):
        self._q = queue.Queue(maxsize=max_pending)
        self._thread = None
        self._err = None

    def submit(self, job):
        if self._thread is None:
            self._thread = threading.Thread(target=self._run, name="frame-writer", daemon=True)
            self._thread.start()
        self._q.put(job)

    def _run(self):
        while True:
            job = self._q.get()
            try:
                job()
            except BaseException as e:  # reported by flush
                if self._err is None:
                    self._err = e
            finally:
                self._q.task_done()

    def flush(self):
        self._q.join()
        if self._err is not None:
            err, self._err = self._err, None
            raise err


class _FrameSlot:
    """One frame in flight from a CUDA device: a device snapshot of positions and
    velocities (taken on the solver's stream, so the next substep may overwrite
    the particle arrays at once), pinned host buffers, and the side stream's
    copy event that the writer waits on."""

    def __init__(self, n, dim, device):
        import torch
        self.dev = torch.empty((2, n, dim), dtype=torch.float32, device=device)
        self.host = torch.empty((2, n, dim), dtype=torch.float32, pin_memory=True)
        self.done = None


class _AsyncFrames:
    """Device-to-host copies of frames that do not synchronise the solver's
    stream: a device-to-device snapshot on the solver's stream (microseconds),
    then the device-to-host copy on a side stream, which the writer thread waits
    for by its event.  Up to ``slots`` frames are in flight; a new frame reuses a
    slot once that slot's files are written."""

    def __init__(self, device, slots=3):
        import torch
        self.device = device
        self.stream = torch.cuda.Stream(device=device)
        self.free = queue.Queue()
        self.slots = slots
        self.made = 0

    def _take(self, n, dim):
        try:
            slot = self.free.get_nowait()
        except queue.Empty:
            if self.made < self.slots:
                self.made += 1
                return _FrameSlot(n, dim, self.device)
            slot = self.free.get()
        if slot.dev.shape[1] < n or slot.dev.shape[2] != dim:
            slot = _FrameSlot(n, dim, self.device)  # the particle count outgrew it
        return slot

    def snapshot(self, pos, vel):
        """Enqueues the copies; returns (slot, host views of pos and vel)."""
        import torch
        n, dim = pos.shape
        slot = self._take(n, dim)
        main = torch.cuda.current_stream(self.device)
        slot.dev[0, :n].copy_(pos)
        slot.dev[1, :n].copy_(vel)
        self.stream.wait_stream(main)
        with torch.cuda.stream(self.stream):
            slot.host[:, :n].copy_(slot.dev[:, :n], non_blocking=True)
            slot.done = torch.cuda.Event()
            slot.done.record(self.stream)
        return slot, slot.host[0, :n], slot.host[1, :n]

    def release(self, slot):
        self.free.put(slot)


class Simulation:
    """The reference's module-level state of ``main.py`` as one object."""

    def __init__(self, config, fbm=False, use_graph=True, device=None, out_dir=None, wcsph=False, map_grid=False):
        self.config = config
        self.ngrid = Ngrid(config)
        self.fluid = Fluid(config.fluid_max_part_num[None], config, uid=0, device=device)
        self.bound = Fluid(config.bound_max_part_num[None], config, uid=1, device=device)
        self.globalvar = GlobalVariable()
        self.scenario_wait_buffer = []
        self.inlets = []
        self.fbm = fbm
        self.wcsph = wcsph
        self.use_graph = use_graph
        # the particle-to-grid map the reference ships commented out (main.py:254)
        self.grid = Grid(config, device=device) if map_grid else None
        self.out_dir = out_dir or config.solver_type
        self._solver = None
        self._writer = None
        self._frames = None

    @property
    def solver(self):
        if self._solver is None:
            self._solver = Solver(self.config, self.fluid, self.bound, fbm=self.fbm, use_graph=self.use_graph,
                                  wcsph=self.wcsph, ngrid=self.ngrid)
        return self._solver

    # ---------------------------------------------------------------- scenario
    def get_obj_from_str(self, s):
        """``main.py:16-23``."""
        if s == "fluid":
            return self.fluid
        if s == "bound":
            return self.bound
        print("scenario WARNING: object does not exist (name:", s, ")")
        return None

    def inlet_helper_get_dt(self, norm, speed, relaxing_factor):
        """``main.py:26-39``."""
        norm = np.array(norm) / np.linalg.norm(np.array(norm))
        if speed < 0:
            norm, speed = -norm, -speed
        acc = np.dot(norm, self.config.gravity[None].astype(np.float64))
        r = float(self.config.part_size[1])
        if acc < 1e-6:
            if speed > 0:
                return r * relaxing_factor / speed
            return float("inf")
        return ((speed ** 2 + 2 * acc * r) ** 0.5 - speed) / acc * relaxing_factor

    def add_to_scenario(self, obj_str, param):
        """``main.py:42-60``."""
        obj = self.get_obj_from_str(obj_str)
        if obj is None:
            print("scenario WARNING: obj '", obj_str, "' non-exist.")
            return
        t = param["type"]
        if t == "cube":
            obj.scene_add_cube(param["start_pos"], param["end_pos"], param["volume_frac"], param["vel"],
                               int(param["color"], 16), param["particle_relaxing_factor"])
        elif t == "box":
            obj.scene_add_box(param["start_pos"], param["end_pos"], param["layers"], param["volume_frac"],
                              param["vel"], int(param["color"], 16), param["particle_relaxing_factor"])
        elif t == "ply":
            verts = read_ply(param["file_name"].replace("\\", os.sep))
            obj.push_part_from_ply(len(verts), verts, param["volume_frac"], param["vel"], int(param["color"], 16))
        elif t == "inlet":
            if np.linalg.norm(np.array(param["norm"])) < 1e-6:
                raise Exception("inlet ERROR: magnitute of attribute 'norm' should not be zero.")
            param["obj"] = obj_str
            param["dt"] = self.inlet_helper_get_dt(param["norm"], param["speed"], param["particle_relaxing_factor"])
            param["t_pre"] = self.globalvar.time_count - param["dt"]
            self.inlets.append(param)

    def init_scenario(self):
        """``main.py:62-79`` (the GGUI-only calls are dropped)."""
        try:
            for part in self.config.scenario_buffer:
                if part != "sim_env":
                    for param in self.config.scenario_buffer[part]["objs"]:
                        if "time" not in param or param["time"] <= 0.0:
                            self.add_to_scenario(part, param)
                        else:
                            param["_part"] = part
                            self.scenario_wait_buffer.append(param)
        except Exception as e:
            raise Exception("scenario ERROR: no scenario file or scenario file invalid.") from e

    def refresh_inlets(self):
        """``main.py:81-100``."""
        gv = self.globalvar
        for i in range(len(self.inlets) - 1, -1, -1):
            inlet = self.inlets[i]
            if "end_time" in inlet and gv.time_count >= inlet["end_time"]:
                self.inlets.pop(i)
            elif gv.time_count >= inlet["t_pre"] + inlet["dt"]:
                try:
                    inlet["t_pre"] = gv.time_count
                    self.get_obj_from_str(inlet["obj"]).scene_add_from_inlet(
                        inlet["center"], inlet["size"], inlet["norm"], inlet["speed"], inlet["volume_frac"],
                        int(inlet["color"], 16), inlet["particle_relaxing_factor"])
                except Exception:
                    warn("inlet WARNING: refresh_inlets failed for:", json.dumps(inlet))
                    self.inlets.pop(i)

    def refresh_scenario(self):
        """``main.py:102-112``."""
        for i in range(len(self.scenario_wait_buffer) - 1, -1, -1):
            param = self.scenario_wait_buffer[i]
            try:
                if param["time"] <= self.globalvar.time_count:
                    self.add_to_scenario(param["_part"], param)
                    self.scenario_wait_buffer.pop(i)
            except Exception:
                warn("scenario WARNING: invalid scenario object:", json.dumps(param))
                self.scenario_wait_buffer.pop(i)
        self.refresh_inlets()

    # ---------------------------------------------------------------- time loop
    def substep(self):
        """One substep of run_step (main.py:347-352): the clock and counters are
        read back once per substep (the time loop needs dt on the host)."""
        self.refresh_scenario()
        s = self.solver
        s.substep()
        if self.grid is not None:
            s.map_velocity(self.grid)
        st = s.stats()
        gv = self.globalvar
        gv.time_count += st["dt"]
        gv.div_iter_count = st["div_iter"]
        gv.incom_iter_count = st["incom_iter"]
        gv.frame_div_iter += gv.div_iter_count
        gv.frame_incom_iter += gv.incom_iter_count
        gv.step_counter += 1
        return st

    def run_step(self, verbose=False):
        """``main.py:339-368``: advance to the next frame at ``gui_fps``."""
        gv = self.globalvar
        gv.time_counter += 1
        while gv.time_count < gv.time_counter / self.config.gui_fps[None]:
            if gv.is_first_time:
                gv.time_start = time.time()
                gv.is_first_time = False
            self.substep()
        gv.time_real = time.time() - gv.time_start
        if verbose:
            print("current time: ", gv.time_count)
            print("---------------------real time------------------------", gv.time_real)
            print("time step: ", self.config.dt[None])

    # ---------------------------------------------------------------- output
    def frame_record(self):
        """Contents of ``write_full_json`` (main.py:151-171)."""
        gv = self.globalvar
        ke = self.fluid.statistics_kinetic_energy[None]
        pe = self.fluid.statistics_gravity_potential_energy[None]
        return {
            "step": gv.step_counter, "frame": gv.time_counter, "timeInSimulation": gv.time_count,
            "timeStep": self.config.dt[None], "fps": self.config.gui_fps[None],
            "iteration": {"divergenceFree_iteration": gv.frame_div_iter,
                          "incompressible_iteration": gv.frame_incom_iter,
                          "sum_iteration": gv.frame_div_iter + gv.frame_incom_iter},
            "energy": {"statistics_kinetic_energy": ke, "statistics_gravity_potential_energy": pe,
                       "sum_energy": ke + pe},
        }

    def write_files(self, wait=True):
        """``main.py:371-378`` without the PNG: PLY of fluid positions, frame JSON,
        npy of positions and velocities.  With ``wait=True`` the frame is copied
        to the host and written before returning.  With ``wait=False`` nothing
        waits for the GPU: on a CUDA device the positions and velocities are
        snapshotted on the solver's stream and copied to pinned host memory on a
        side stream, and a background thread writes the files once that copy has
        finished, while the caller goes on stepping (``flush`` waits for every
        frame)."""
        d = self.config.dim[None]
        n = self.fluid.part_num[None]
        frame = self.globalvar.time_counter
        out = self.out_dir
        rec = json.dumps(self.frame_record())

        def write(pos, vel):
            for sub in ("ply", "json", "part_data"):
                os.makedirs(os.path.join(out, sub), exist_ok=True)
            write_ply(os.path.join(out, "ply", "fluid_pos"), frame, d, n, pos)
            with open(os.path.join(out, "json", "frame%d.json" % frame), "w") as f:
                f.write(rec)
            np.save(os.path.join(out, "part_data", "vel_%d" % frame), vel)
            np.save(os.path.join(out, "part_data", "pos_%d" % frame), pos)

        fpos, fvel = self.fluid.pos[:n].detach(), self.fluid.vel[:n].detach()
        if wait:
            write(fpos.to("cpu", copy=True).numpy(), fvel.to("cpu", copy=True).numpy())
            return
        if self._writer is None:
            self._writer = FrameWriter()
        if fpos.device.type != "cuda":
            pos, vel = fpos.clone().numpy(), fvel.clone().numpy()
            self._writer.submit(lambda: write(pos, vel))
            return
        if self._frames is None:
            self._frames = _AsyncFrames(fpos.device)
        frames = self._frames
        slot, hpos, hvel = frames.snapshot(fpos, fvel)

        def job():
            try:
                slot.done.synchronize()
                write(hpos.numpy(), hvel.numpy())
            finally:
                frames.release(slot)

        self._writer.submit(job)

    def flush(self):
        """Waits until every frame passed to ``write_files(wait=False)`` is on disk."""
        if self._writer is not None:
            self._writer.flush()
