"""ctypes driver of ``oracle/sph_port.c`` -- TEST INFRASTRUCTURE ONLY.

The reference-structured C restatement (OpenMP) in two builds: FP32 (the
reference's arithmetic; the timed CPU baseline and a mid-size cross-check) and
FP64 (``fp64=True``: every sum and pair term in double over the FP32 particle
arrays; the one-step oracle at the benchmark sizes).  Particle arrays are host
numpy arrays laid out exactly like the CUDA path's ``tsph_set`` views.
"""
import ctypes as C
import os

import numpy as np

from tichi_sph_gb300 import _native

HERE = os.path.dirname(os.path.abspath(__file__))


class PortStats(C.Structure):
    _fields_ = [("dt", C.c_double), ("time_count", C.c_double), ("compression", C.c_double),
                ("kinetic_energy", C.c_double), ("potential_energy", C.c_double),
                ("div_iter", C.c_int32), ("incom_iter", C.c_int32), ("fbm_passes", C.c_int32)]


_LIBS = {}


def lib(fp64=False):
    real = "double" if fp64 else "float"
    if real not in _LIBS:
        from oracle import build_oracle
        path = build_oracle.build(real=real)
        L = C.CDLL(path)
        L.port_create.restype = C.c_void_p
        L.port_create.argtypes = [C.POINTER(_native.Params), C.c_int64, C.c_int64]
        L.port_destroy.argtypes = [C.c_void_p]
        L.port_set_state.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.port_substep.restype = C.c_int
        L.port_substep.argtypes = [C.c_void_p, C.POINTER(_native.Set), C.POINTER(_native.Set), C.POINTER(PortStats)]
        L.port_num_threads.restype = C.c_int
        _LIBS[real] = L
    return _LIBS[real]


class HostSet:
    """Host arrays of one particle set (the ``tsph_set`` fields)."""

    def __init__(self, n, dim, P, arrays):
        self.n = n
        z = lambda *s: np.zeros(s, dtype=np.float32)
        self.a = {
            "pos": z(n, dim), "vel": z(n, dim), "vel_adv": z(n, dim), "acce": z(n, dim), "acce_adv": z(n, dim),
            "mass": z(n), "rest_density": z(n), "rest_volume": z(n), "volume_frac": z(n, P),
            "volume_frac_tmp": z(n, P), "W": z(n), "sph_density": z(n), "sph_compression": z(n),
            "psi_adv": z(n), "alpha": z(n), "alpha_1": z(n, dim), "alpha_2": z(n), "normal": z(n, dim),
            "drift_vel": z(n, P, dim), "fbm_zeta": z(n), "pressure": z(n),
            "flag": np.zeros(n, np.int32), "neighb_cell_seq": np.zeros(n, np.int32),
            "neighb_in_cell_seq": np.zeros(n, np.int32), "neighb_cell_structured_seq": np.zeros((n, dim), np.int32),
        }
        for k, v in arrays.items():
            self.a[k][...] = np.asarray(v, dtype=self.a[k].dtype).reshape(self.a[k].shape)
        s = _native.Set()
        s.n = n
        s.capacity = n
        for f in _native.SET_FLOAT_FIELDS:
            setattr(s, f, self.a[f].ctypes.data_as(_native._fp))
        for f in _native.SET_INT_FIELDS:
            setattr(s, f, self.a[f].ctypes.data_as(_native._ip))
        self.s = s

    def __getattr__(self, k):
        a = self.__dict__.get("a")
        if a is not None and k in a:
            return a[k]
        raise AttributeError(k)


class PortSim:
    """The C restatement stepping one (fluid, boundary) pair."""

    def __init__(self, config, fluid_arrays, bound_arrays, fbm=False, fbm_max_passes=1000, fp64=False):
        d, P = config.dim[None], config.phase_num[None]
        self.L = lib(fp64)
        self.fluid = HostSet(len(fluid_arrays["pos"]), d, P, fluid_arrays)
        self.bound = HostSet(len(bound_arrays["pos"]), d, P, bound_arrays)
        self.params = config.to_params(fbm_enabled=fbm, fbm_max_passes=fbm_max_passes)
        self.h = self.L.port_create(C.byref(self.params), self.fluid.n, self.bound.n)
        self.stats = PortStats()

    def set_state(self, time_count=0.0, compression=0.0):
        self.L.port_set_state(self.h, time_count, compression)

    def substep(self):
        self.L.port_substep(self.h, C.byref(self.fluid.s), C.byref(self.bound.s), C.byref(self.stats))
        return {k: getattr(self.stats, k) for k, _ in PortStats._fields_}

    def threads(self):
        return self.L.port_num_threads()

    def close(self):
        if self.h:
            self.L.port_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
