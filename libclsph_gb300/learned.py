"""ctypes binding of the learned 4x-dt stepper (include/clsph_learned.h).

`Mlp` holds the per-particle network (BF16 tensor-core kernels, FP32
accumulation) with its training state; `Collector` records training samples
from plain substeps of a `GpuSolver`; `step_learned` advances a solver with
learned steps under the density check. Device buffers handed to these
functions are plain CUDA pointers (torch tensors are used only as device
memory by the tests and scripts). No counterpart in the reference.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from .gpu import ClsphError, GpuSolver, load_library

_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64

N_FEATURES = 32
N_OUTPUTS = 4
HIDDEN = 256
# blob layout (floats)
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_FEATURES * HIDDEN
OFF_W2 = OFF_B1 + HIDDEN
OFF_B2 = OFF_W2 + HIDDEN * HIDDEN
OFF_W3 = OFF_B2 + HIDDEN
OFF_B3 = OFF_W3 + HIDDEN * N_OUTPUTS
N_PARAMS = OFF_B3 + N_OUTPUTS
OFF_XMU = N_PARAMS
OFF_XSIGMA = OFF_XMU + N_FEATURES
OFF_YMU = OFF_XSIGMA + N_FEATURES
OFF_YSIGMA = OFF_YMU + N_OUTPUTS
BLOB = OFF_YSIGMA + N_OUTPUTS

FEATURE_NAMES = [
    "rho/rho0-1", "p/K", "count/32", "ax", "ay", "az", "vx", "vy", "vz", "|v|/vmax",
    "m1x", "m1y", "m1z", "mxx", "myy", "mzz", "mxy", "mxz", "myz",
    "u1x", "u1y", "u1z", "uxx", "uyy", "uzz", "uxy", "uxz", "uyz", "div", "curlx", "curly", "curlz",
]


class TrainConfig(ctypes.Structure):
    _fields_ = [("epochs", _u32), ("batch", _u32), ("lr", ctypes.c_float), ("lr_final", ctypes.c_float),
                ("seed", _u64), ("fit_normalisation", ctypes.c_int), ("log_every", _u32)]


CALIBRATE = 1  # CLSPH_LEARNED_CALIBRATE
NO_CHECK = 2  # CLSPH_LEARNED_NO_CHECK


class LearnedConfig(ctypes.Structure):
    _fields_ = [("dt_mult", _u32), ("threshold", ctypes.c_float), ("flags", _u32)]


class LearnedStats(ctypes.Structure):
    _fields_ = [("learned_steps", _u64), ("rejected", _u64), ("plain_substeps", _u64), ("checks", _u64),
                ("deviation_sum", ctypes.c_double), ("deviation_max", ctypes.c_double),
                ("particle_deviation_sum", ctypes.c_double), ("calibration_d", ctypes.c_double),
                ("calibration_m", ctypes.c_double)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["deviation_mean"] = self.deviation_sum / self.checks if self.checks else 0.0
        d["particle_deviation_mean"] = self.particle_deviation_sum / self.checks if self.checks else 0.0
        total = self.learned_steps + self.rejected
        d["fallback_fraction"] = self.rejected / total if total else 0.0
        return d


# (name, restype, argtypes) of every symbol include/clsph_learned.h declares
SIGNATURES = [
    ("clsph_mlp_blob_size", _u64, []),
    ("clsph_mlp_create", ctypes.c_int, [_u64, ctypes.POINTER(_vp)]),
    ("clsph_mlp_destroy", ctypes.c_int, [_vp]),
    ("clsph_mlp_set_blob", ctypes.c_int, [_vp, _vp, _u64]),
    ("clsph_mlp_get_blob", ctypes.c_int, [_vp, _vp, _u64]),
    ("clsph_mlp_forward", ctypes.c_int, [_vp, _vp, _u32, _vp, _vp]),
    ("clsph_mlp_forward_mma_sync", ctypes.c_int, [_vp, _vp, _u32, _vp, _vp]),
    ("clsph_mlp_status", ctypes.c_int, [_vp, ctypes.POINTER(_u32)]),
    ("clsph_mlp_predict", ctypes.c_int, [_vp, _vp, _u64, _vp]),
    ("clsph_mlp_gradients", ctypes.c_int, [_vp, _vp, _vp, _u32, _vp, ctypes.POINTER(ctypes.c_float)]),
    ("clsph_mlp_train", ctypes.c_int,
     [_vp, _vp, _vp, _u64, ctypes.POINTER(TrainConfig), _vp, _u32, ctypes.POINTER(_u32)]),
    ("clsph_mlp_loss", ctypes.c_int, [_vp, _vp, _vp, _u64, ctypes.POINTER(ctypes.c_float)]),
    ("clsph_collector_create", ctypes.c_int, [_vp, _u32, _u32, _u64, ctypes.POINTER(_vp)]),
    ("clsph_collector_destroy", ctypes.c_int, [_vp]),
    ("clsph_collector_step", ctypes.c_int, [_vp, _u32]),
    ("clsph_collector_step_learned", ctypes.c_int, [_vp, _vp, _u32]),
    ("clsph_collector_samples", ctypes.c_int,
     [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_u64)]),
    ("clsph_collector_copy", ctypes.c_int, [_vp, _vp, _vp, _u64, _u64]),
    ("clsph_gpu_read_features", ctypes.c_int, [_vp, _vp]),
    ("clsph_gpu_step_learned", ctypes.c_int,
     [_vp, _vp, _u32, ctypes.POINTER(LearnedConfig), ctypes.POINTER(LearnedStats)]),
]

_BOUND = False


def library() -> ctypes.CDLL:
    global _BOUND
    lib = load_library()
    if not _BOUND:
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _BOUND = True
    return lib


def _check(lib, fn: str, code: int) -> None:
    if code != 0:
        raise ClsphError(fn, code, (lib.clsph_gpu_last_error() or b"").decode(errors="replace"))


def default_weights_path() -> Path:
    return Path(__file__).resolve().parent / "weights" / "stepper_4dt.npz"


class Mlp:
    """The stepper's network on the current CUDA device."""

    def __init__(self, seed: int = 0, blob: np.ndarray | None = None):
        self.lib = library()
        assert self.lib.clsph_mlp_blob_size() == BLOB
        h = _vp()
        _check(self.lib, "clsph_mlp_create", self.lib.clsph_mlp_create(seed, ctypes.byref(h)))
        self.h = h
        if blob is not None:
            self.set_blob(blob)

    @classmethod
    def load(cls, path: str | Path | None = None) -> "Mlp":
        path = Path(path) if path is not None else default_weights_path()
        with np.load(path) as z:
            return cls(blob=np.asarray(z["blob"], dtype=np.float32))

    def save(self, path: str | Path, **meta) -> None:
        np.savez_compressed(path, blob=self.blob(), **meta)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.clsph_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def blob(self) -> np.ndarray:
        out = np.empty(BLOB, dtype=np.float32)
        _check(self.lib, "clsph_mlp_get_blob", self.lib.clsph_mlp_get_blob(self.h, out.ctypes.data, BLOB))
        return out

    def set_blob(self, blob: np.ndarray) -> None:
        b = np.ascontiguousarray(blob, dtype=np.float32)
        if b.size != BLOB:
            raise ValueError(f"blob has {b.size} floats, expected {BLOB}")
        _check(self.lib, "clsph_mlp_set_blob", self.lib.clsph_mlp_set_blob(self.h, b.ctypes.data, BLOB))

    def forward(self, x_bf16_ptr: int, rows: int, y_ptr: int, stream: int = 0) -> None:
        """Fused inference on device buffers (standardised bf16 rows -> float4 rows)."""
        _check(self.lib, "clsph_mlp_forward",
               self.lib.clsph_mlp_forward(self.h, x_bf16_ptr, rows, y_ptr, stream or None))

    def forward_mma_sync(self, x_bf16_ptr: int, rows: int, y_ptr: int, stream: int = 0) -> None:
        """The same inference on the warp-level mma.sync path (cross-check)."""
        _check(self.lib, "clsph_mlp_forward_mma_sync",
               self.lib.clsph_mlp_forward_mma_sync(self.h, x_bf16_ptr, rows, y_ptr, stream or None))

    def predict(self, x_ptr: int, rows: int) -> np.ndarray:
        """Predictions [rows][4] (host) for raw device feature rows."""
        y = np.empty((rows, N_OUTPUTS), dtype=np.float32)
        _check(self.lib, "clsph_mlp_predict", self.lib.clsph_mlp_predict(self.h, x_ptr, rows, y.ctypes.data))
        return y

    def status(self) -> int:
        """Error bits of the tensor-core inference since the last call (0 = none)."""
        f = _u32()
        _check(self.lib, "clsph_mlp_status", self.lib.clsph_mlp_status(self.h, ctypes.byref(f)))
        return int(f.value)

    def gradients(self, x_ptr: int, y_ptr: int, rows: int) -> tuple[np.ndarray, float]:
        g = np.empty(N_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        _check(self.lib, "clsph_mlp_gradients",
               self.lib.clsph_mlp_gradients(self.h, x_ptr, y_ptr, rows, g.ctypes.data, ctypes.byref(loss)))
        return g, float(loss.value)

    def loss(self, x_ptr: int, y_ptr: int, samples: int) -> float:
        out = ctypes.c_float()
        _check(self.lib, "clsph_mlp_loss", self.lib.clsph_mlp_loss(self.h, x_ptr, y_ptr, samples, ctypes.byref(out)))
        return float(out.value)

    def train(self, x_ptr: int, y_ptr: int, samples: int, epochs: int = 1, batch: int = 65536,
              lr: float = 1e-3, lr_final: float = 1e-4, seed: int = 0, fit_normalisation: bool = True,
              log_every: int = 50) -> np.ndarray:
        cfg = TrainConfig(epochs, batch, lr, lr_final, seed, 1 if fit_normalisation else 0, log_every)
        log = np.zeros(4096, dtype=np.float32)
        n = _u32()
        _check(self.lib, "clsph_mlp_train",
               self.lib.clsph_mlp_train(self.h, x_ptr, y_ptr, samples, ctypes.byref(cfg), log.ctypes.data,
                                        len(log), ctypes.byref(n)))
        return log[: n.value].copy()


class Collector:
    """Training samples from plain substeps of `solver` (same trajectory as solver.step)."""

    def __init__(self, solver: GpuSolver, id_stride: int, capacity: int, dt_mult: int = 4):
        self.lib = library()
        h = _vp()
        _check(self.lib, "clsph_collector_create",
               self.lib.clsph_collector_create(solver.h, id_stride, dt_mult, capacity, ctypes.byref(h)))
        self.h = h
        self.solver = solver

    def step(self, substeps: int) -> None:
        _check(self.lib, "clsph_collector_step", self.lib.clsph_collector_step(self.h, substeps))

    def step_learned(self, mlp: "Mlp", steps: int) -> None:
        """Learned steps with `mlp`, recording the plain outcome of every visited state."""
        _check(self.lib, "clsph_collector_step_learned", self.lib.clsph_collector_step_learned(self.h, mlp.h, steps))

    def samples(self) -> tuple[int, int, int]:
        """(x device pointer, y device pointer, count)."""
        x, y, n = _vp(), _vp(), _u64()
        _check(self.lib, "clsph_collector_samples",
               self.lib.clsph_collector_samples(self.h, ctypes.byref(x), ctypes.byref(y), ctypes.byref(n)))
        return int(x.value or 0), int(y.value or 0), int(n.value)

    def copy(self, first: int = 0, count: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        """Host copies of samples [first, first + count): x [count][32], y [count][4]."""
        total = self.samples()[2]
        count = total - first if count is None else count
        x = np.empty((count, N_FEATURES), dtype=np.float32)
        y = np.empty((count, N_OUTPUTS), dtype=np.float32)
        _check(self.lib, "clsph_collector_copy",
               self.lib.clsph_collector_copy(self.h, x.ctypes.data, y.ctypes.data, first, count))
        return x, y

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.clsph_collector_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_features(solver: GpuSolver) -> np.ndarray:
    lib = library()
    out = np.empty((solver.n, N_FEATURES), dtype=np.float32)
    _check(lib, "clsph_gpu_read_features", lib.clsph_gpu_read_features(solver.h, out.ctypes.data))
    return out


def step_learned(solver: GpuSolver, mlp: Mlp, steps: int, dt_mult: int = 4, threshold: float = 0.01,
                 stats: LearnedStats | None = None, calibrate: bool = False,
                 check: bool = True) -> LearnedStats:
    """clsph_gpu_step_learned; check=False runs the steps back to back without
    the density check (threshold ignored)."""
    lib = library()
    st = stats if stats is not None else LearnedStats()
    cfg = LearnedConfig(dt_mult, threshold, (CALIBRATE if calibrate else 0) | (0 if check else NO_CHECK))
    _check(lib, "clsph_gpu_step_learned",
           lib.clsph_gpu_step_learned(solver.h, mlp.h, steps, ctypes.byref(cfg), ctypes.byref(st)))
    return st
