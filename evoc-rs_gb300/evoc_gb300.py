"""ctypes binding of libevoc_gb300.so (the C ABI in include/evoc_gb300.h).

The binding mirrors the Rust functions the library replaces in evoc-rs 0.2.7:

    build_fuzzy_simplicial_set   src/graph/fuzzy_graph.rs:275-295
    coo_to_adjacency_list        src/graph/fuzzy_graph.rs:242-256
    smooth_knn_dist              src/graph/fuzzy_graph.rs:33-98
    evoc_embedding               src/graph/embedding.rs:48-298
    EvocEmbeddingParams          src/graph/mod.rs:22-67
    label_propagation_init       src/graph/label_prop.rs:537-564
    build_mst                    src/clustering/mst.rs:82-166

There is no CPU fallback: importing works anywhere, but creating a Context
raises EvocError when the shared library or an sm_103 GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("EVOC_GB300_LIB", _HERE / "libevoc_gb300.so"))

EVOC_OK = 0
EVOC_ERR_INVALID_ARGUMENT = -1
EVOC_ERR_INVALID_INPUT = -2
EVOC_ERR_UNSUPPORTED = -3
EVOC_ERR_CUDA = -4
EVOC_ERR_OUT_OF_MEMORY = -5
EVOC_ERR_NO_DEVICE = -6
EVOC_ERR_INTERNAL = -7
KNN_PAD = 0xFFFFFFFF
NOALLOC_SCRATCH_BYTES = 16 << 20  # EVOC_NOALLOC_SCRATCH_BYTES

# Every symbol declared in include/evoc_gb300.h.
EXPORTED = [
    "evoc_abi_version", "evoc_embed_params_default", "evoc_ctx_create",
    "evoc_ctx_destroy", "evoc_last_error", "evoc_ctx_stream", "evoc_smooth_knn_dist",
    "evoc_fuzzy_set", "evoc_fuzzy_set_device", "evoc_graph_from_csr",
    "evoc_graph_info", "evoc_graph_export", "evoc_graph_free", "evoc_embed",
    "evoc_plan_create", "evoc_plan_run_device", "evoc_plan_enqueue_device",
    "evoc_plan_profile_epochs", "evoc_plan_info", "evoc_plan_stats",
    "evoc_plan_debug_run", "evoc_plan_free", "evoc_embed_batched",
    "evoc_knn_to_csr_noalloc", "evoc_gather_peak", "evoc_plan_create_batched",
    "evoc_fuzzy_set_batched", "evoc_plan_create_blocks", "evoc_embed_blocks",
    "evoc_mlp_train_params_default", "evoc_mlp_create", "evoc_mlp_free",
    "evoc_mlp_n_params", "evoc_mlp_get_params", "evoc_mlp_set_params", "evoc_mlp_predict",
    "evoc_mlp_predict_device", "evoc_mlp_gradients", "evoc_mlp_fit_device",
    "evoc_to_bf16_device", "evoc_procrustes", "evoc_fuzzy_set_device_raw",
    "evoc_label_prop_partition", "evoc_selftest_wait_timeout", "evoc_ctx_smooth_knn_steps",
    "evoc_plan_set_config", "evoc_plan_autotune", "evoc_label_propagation_init",
    "evoc_label_propagation_init_device", "evoc_build_mst", "evoc_build_mst_device",
]


class EvocError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class EmbedParamsC(C.Structure):
    _fields_ = [
        ("n_epochs", C.c_int32),
        ("noise_level", C.c_float),
        ("negative_sample_rate", C.c_float),
        ("initial_alpha", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("eps", C.c_float),
    ]


class MlpTrainParamsC(C.Structure):
    _fields_ = [
        ("steps", C.c_int32),
        ("batch", C.c_int32),
        ("align_every", C.c_int32),
        ("align_rows", C.c_int32),
        ("lr", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("eps", C.c_float),
        ("lr_end", C.c_float),
        ("seed", C.c_uint64),
    ]


@dataclass
class MlpTrainParams:
    """evoc_mlp_train_params_t with its defaults."""
    steps: int = 3000
    batch: int = 8192
    align_every: int = 250
    align_rows: int = 65536
    lr: float = 1e-3
    beta1: float = 0.9
    beta2: float = 0.999
    eps: float = 1e-8
    lr_end: float = 1e-4
    seed: int = 0

    def to_c(self) -> MlpTrainParamsC:
        return MlpTrainParamsC(int(self.steps), int(self.batch), int(self.align_every),
                               int(self.align_rows), self.lr, self.beta1, self.beta2,
                               self.eps, self.lr_end, int(self.seed))


class EpochStatsC(C.Structure):
    _fields_ = [("fired_edges", C.c_int64), ("negatives", C.c_int64),
                ("active_nodes", C.c_int64)]


@dataclass
class EvocEmbeddingParams:
    """Mirror of EvocEmbeddingParams (src/graph/mod.rs:22-67) with its defaults."""
    n_epochs: int = 50
    noise_level: float = 0.5
    negative_sample_rate: float = 1.0
    initial_alpha: float = 0.1
    beta1: float = 0.5
    beta2: float = 0.9
    eps: float = 1e-7

    def to_c(self) -> EmbedParamsC:
        return EmbedParamsC(int(self.n_epochs), self.noise_level,
                            self.negative_sample_rate, self.initial_alpha,
                            self.beta1, self.beta2, self.eps)


_lib = None


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Load the shared library and declare its signatures (no GPU needed)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise EvocError(EVOC_ERR_NO_DEVICE,
                        f"{p} not found: build it with python evoc-rs_gb300/build.py")
    lib = C.CDLL(str(p))
    vp, i32, i64, u64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_float
    pp = C.POINTER(C.c_void_p)
    sig = {
        "evoc_abi_version": ([], C.c_int),
        "evoc_embed_params_default": ([C.POINTER(EmbedParamsC)], None),
        "evoc_ctx_create": ([C.c_int, pp], C.c_int),
        "evoc_ctx_destroy": ([vp], None),
        "evoc_last_error": ([vp], C.c_char_p),
        "evoc_ctx_stream": ([vp], C.c_void_p),
        "evoc_ctx_smooth_knn_steps": ([vp, C.POINTER(C.c_int64)], C.c_int),
        "evoc_plan_set_config": ([vp, C.c_int32, C.c_int32, C.c_int32], C.c_int),
        "evoc_plan_autotune": ([vp, vp, C.POINTER(C.c_float)], C.c_int),
        "evoc_label_propagation_init": ([vp, vp, C.c_int32, vp, C.c_int64, C.c_uint64, vp],
                                        C.c_int),
        "evoc_label_propagation_init_device": ([vp, vp, C.c_int32, vp, C.c_int64, C.c_uint64,
                                               vp], C.c_int),
        "evoc_build_mst": ([vp, vp, C.c_int64, C.c_int32, C.c_int32, vp, vp, vp,
                            C.POINTER(C.c_int64)], C.c_int),
        "evoc_build_mst_device": ([vp, vp, C.c_int64, C.c_int32, C.c_int32, vp, vp, vp,
                                   C.POINTER(C.c_int64)], C.c_int),
        "evoc_smooth_knn_dist": ([vp, vp, vp, i64, i32, u64, f32, i32, vp, vp], C.c_int),
        "evoc_fuzzy_set": ([vp, vp, vp, i64, i32, f32, C.c_int, pp], C.c_int),
        "evoc_fuzzy_set_device": ([vp, vp, vp, i64, i32, f32, C.c_int, vp, vp, pp], C.c_int),
        "evoc_fuzzy_set_device_raw": ([vp, vp, vp, i64, i32, i32, f32, C.c_int, pp], C.c_int),
        "evoc_label_prop_partition": ([vp, vp, i64, i32, u64, vp, C.POINTER(i64)], C.c_int),
        "evoc_selftest_wait_timeout": ([vp, i32], C.c_int),
        "evoc_graph_from_csr": ([vp, vp, vp, vp, i64, pp], C.c_int),
        "evoc_graph_info": ([vp, C.POINTER(i64), C.POINTER(i64)], C.c_int),
        "evoc_graph_export": ([vp, vp, vp, vp], C.c_int),
        "evoc_graph_free": ([vp], None),
        "evoc_embed": ([vp, vp, i32, C.POINTER(EmbedParamsC), vp, u64, i32, vp], C.c_int),
        "evoc_plan_create": ([vp, vp, i32, C.POINTER(EmbedParamsC), u64, pp], C.c_int),
        "evoc_plan_run_device": ([vp, vp, vp], C.c_int),
        "evoc_plan_enqueue_device": ([vp, vp, vp], C.c_int),
        "evoc_plan_profile_epochs": ([vp, vp, vp, vp], C.c_int),
        "evoc_gather_peak": ([vp, i64, C.POINTER(C.c_double)], C.c_int),
        "evoc_plan_create_batched": ([vp, i32, vp, i32, vp, vp, pp], C.c_int),
        "evoc_fuzzy_set_batched": ([vp, i32, vp, vp, vp, i32, f32, C.c_int, pp], C.c_int),
        "evoc_plan_create_blocks": ([vp, vp, i32, vp, i32, vp, vp, pp], C.c_int),
        "evoc_embed_blocks": ([vp, vp, i32, vp, i32, vp, vp, vp, vp], C.c_int),
        "evoc_plan_info": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i32),
                            C.POINTER(i32), C.POINTER(i64)], C.c_int),
        "evoc_plan_stats": ([vp, C.POINTER(EpochStatsC)], C.c_int),
        "evoc_plan_debug_run": ([vp, vp, i32, i32, vp, vp], C.c_int),
        "evoc_plan_free": ([vp], None),
        "evoc_embed_batched": ([vp, i32, vp, i32, C.POINTER(EmbedParamsC), vp, vp, vp], C.c_int),
        "evoc_knn_to_csr_noalloc": ([vp, vp, i64, i32, f32, vp, vp, vp, i64, C.POINTER(i64), vp],
                                    C.c_int),
        "evoc_mlp_train_params_default": ([C.POINTER(MlpTrainParamsC)], None),
        "evoc_mlp_create": ([vp, i32, i32, i32, u64, pp], C.c_int),
        "evoc_mlp_free": ([vp], None),
        "evoc_mlp_n_params": ([vp], i64),
        "evoc_mlp_get_params": ([vp, vp], C.c_int),
        "evoc_mlp_set_params": ([vp, vp], C.c_int),
        "evoc_mlp_predict": ([vp, vp, i64, vp], C.c_int),
        "evoc_mlp_predict_device": ([vp, vp, i64, vp], C.c_int),
        "evoc_mlp_gradients": ([vp, vp, vp, i64, vp, vp], C.c_int),
        "evoc_mlp_fit_device": ([vp, i32, vp, vp, vp, C.POINTER(MlpTrainParamsC), vp], C.c_int),
        "evoc_to_bf16_device": ([vp, vp, i64, vp], C.c_int),
        "evoc_procrustes": ([vp, i32, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.evoc_abi_version() != 1:
        raise EvocError(EVOC_ERR_INTERNAL, "ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class Graph:
    """Device-resident weighted adjacency list (evoc_graph_t)."""

    def __init__(self, ctx: "Context", handle: C.c_void_p):
        self._ctx = ctx
        self.handle = handle
        ctx._children.add(self)

    @property
    def n(self) -> int:
        return self.info()[0]

    @property
    def nnz(self) -> int:
        return self.info()[1]

    def info(self) -> tuple[int, int]:
        n, nnz = C.c_int64(), C.c_int64()
        self._ctx._check(self._ctx.lib.evoc_graph_info(self.handle, C.byref(n), C.byref(nnz)))
        return n.value, nnz.value

    def export(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n, nnz = self.info()
        indptr = np.zeros(n + 1, dtype=np.int64)
        indices = np.zeros(nnz, dtype=np.uint32)
        weights = np.zeros(nnz, dtype=np.float32)
        self._ctx._check(self._ctx.lib.evoc_graph_export(
            self.handle, _ptr(indptr), _ptr(indices), _ptr(weights)))
        return indptr, indices, weights

    def to_coo(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """CoordinateList form: (row_indices, col_indices, values)."""
        indptr, indices, weights = self.export()
        rows = np.repeat(np.arange(len(indptr) - 1, dtype=np.int64), np.diff(indptr))
        return rows, indices.astype(np.int64), weights

    def free(self) -> None:
        if self.handle and self._ctx.handle:  # a closed context freed it already
            self._ctx.lib.evoc_graph_free(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Plan:
    """Per-graph set-up of evoc_embedding, reusable across runs (evoc_plan_t)."""

    def __init__(self, ctx: "Context", handle, n: int, dim: int, n_epochs: int):
        self._ctx = ctx
        self.handle = handle
        ctx._children.add(self)
        self.n, self.dim, self.n_epochs = n, dim, n_epochs

    def run_device(self, d_init: int | None, d_out: int) -> None:
        self._ctx._check(self._ctx.lib.evoc_plan_run_device(
            self.handle, C.c_void_p(d_init) if d_init else None, C.c_void_p(d_out)))

    def enqueue_device(self, d_init: int | None, d_out: int) -> None:
        """Enqueue the epoch loop on the context stream without waiting."""
        self._ctx._check(self._ctx.lib.evoc_plan_enqueue_device(
            self.handle, C.c_void_p(d_init) if d_init else None, C.c_void_p(d_out)))

    def profile_epochs(self, d_init: int | None, d_out: int) -> np.ndarray:
        """Device milliseconds of each epoch launch (separate launches, events between)."""
        ms = np.zeros(max(self.n_epochs, 1), dtype=np.float32)
        self._ctx._check(self._ctx.lib.evoc_plan_profile_epochs(
            self.handle, C.c_void_p(d_init) if d_init else None, C.c_void_p(d_out), _ptr(ms)))
        return ms[: self.n_epochs]

    def info(self) -> dict:
        e, i, p, l, r = C.c_int64(), C.c_int64(), C.c_int32(), C.c_int32(), C.c_int64()
        self._ctx._check(self._ctx.lib.evoc_plan_info(self.handle, C.byref(e), C.byref(i),
                                                      C.byref(p), C.byref(l), C.byref(r)))
        return {"n_edges": e.value, "n_incidence": i.value, "neg_planes": p.value,
                "warps_per_block": l.value, "n_slots": r.value}

    def set_config(self, variant: int, warps_per_block: int, blocks_per_sm: int = 0) -> None:
        """Epoch-kernel configuration (identical results for every choice)."""
        self._ctx._check(self._ctx.lib.evoc_plan_set_config(self.handle, int(variant),
                                                             int(warps_per_block),
                                                             int(blocks_per_sm)))

    def autotune(self) -> dict:
        """Pick the fastest epoch-kernel configuration for this plan's shape
        (cached per shape); returns it with its time per epoch launch."""
        cfg = np.zeros(3, dtype=np.int32)
        ms = C.c_float()
        self._ctx._check(self._ctx.lib.evoc_plan_autotune(self.handle, _ptr(cfg), C.byref(ms)))
        return {"variant": int(cfg[0]), "warps_per_block": int(cfg[1]),
                "blocks_per_sm": int(cfg[2]), "ms_per_launch": round(float(ms.value), 4)}

    def stats(self) -> np.ndarray:
        arr = (EpochStatsC * max(self.n_epochs, 1))()
        self._ctx._check(self._ctx.lib.evoc_plan_stats(self.handle, arr))
        out = np.zeros((self.n_epochs, 3), dtype=np.int64)
        for t in range(self.n_epochs):
            out[t] = (arr[t].fired_edges, arr[t].negatives, arr[t].active_nodes)
        return out

    def debug_run(self, init: np.ndarray | None, start_epoch: int, end_epoch: int,
                  want_grad: bool = False):
        out = np.zeros((self.n, self.dim), dtype=np.float32)
        grad = np.zeros((self.n, self.dim), dtype=np.float32) if want_grad else None
        init_c = None if init is None else _f32(init)
        self._ctx._check(self._ctx.lib.evoc_plan_debug_run(
            self.handle, _ptr(init_c), start_epoch, end_epoch, _ptr(out), _ptr(grad)))
        return (out, grad) if want_grad else out

    def free(self) -> None:
        if self.handle and self._ctx.handle:  # a closed context freed it already
            self._ctx.lib.evoc_plan_free(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Mlp:
    """The learned warm start (evoc_mlp_t): in_dim -> hidden -> hidden -> out_dim."""

    def __init__(self, ctx: "Context", handle, in_dim: int, hidden: int, out_dim: int):
        self._ctx = ctx
        self.handle = handle
        ctx._children.add(self)
        self.in_dim, self.hidden, self.out_dim = in_dim, hidden, out_dim

    @property
    def n_params(self) -> int:
        return int(self._ctx.lib.evoc_mlp_n_params(self.handle))

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        self._ctx._check(self._ctx.lib.evoc_mlp_get_params(self.handle, _ptr(out)))
        return out

    def set_params(self, params) -> None:
        p = _f32(params)
        if p.shape != (self.n_params,):
            raise ValueError(f"expected {self.n_params} parameters")
        self._ctx._check(self._ctx.lib.evoc_mlp_set_params(self.handle, _ptr(p)))

    def unpack(self, flat: np.ndarray) -> dict:
        """Split a packed parameter (or gradient) array into named arrays."""
        i, h, o = self.in_dim, self.hidden, self.out_dim
        sizes = [("w1", (h, i)), ("b1", (h,)), ("w2", (h, h)), ("b2", (h,)),
                 ("w3", (o, h)), ("b3", (o,))]
        out, at = {}, 0
        for name, shape in sizes:
            cnt = int(np.prod(shape))
            out[name] = flat[at:at + cnt].reshape(shape)
            at += cnt
        return out

    def predict(self, x) -> np.ndarray:
        xx = _f32(x)
        n = xx.shape[0]
        out = np.zeros((n, self.out_dim), dtype=np.float32)
        self._ctx._check(self._ctx.lib.evoc_mlp_predict(self.handle, _ptr(xx), n, _ptr(out)))
        return out

    def predict_device(self, d_x_bf16: int, n: int, d_out: int) -> None:
        self._ctx._check(self._ctx.lib.evoc_mlp_predict_device(
            self.handle, C.c_void_p(d_x_bf16), int(n), C.c_void_p(d_out)))

    def gradients(self, x, target) -> tuple[float, np.ndarray]:
        xx, tt = _f32(x), _f32(target)
        loss = np.zeros(1, dtype=np.float32)
        grad = np.zeros(self.n_params, dtype=np.float32)
        self._ctx._check(self._ctx.lib.evoc_mlp_gradients(
            self.handle, _ptr(xx), _ptr(tt), xx.shape[0], _ptr(loss), _ptr(grad)))
        return float(loss[0]), grad

    def fit_device(self, d_points_bf16: Sequence[int], d_layouts: Sequence[int],
                   n_rows: Sequence[int], params: MlpTrainParams | None = None) -> np.ndarray:
        """Train on device-resident (BF16 points, f32 layout) instances; returns
        the per-step mean squared error."""
        p = (params or MlpTrainParams()).to_c()
        m = len(n_rows)
        xh = (C.c_void_p * m)(*[int(a) for a in d_points_bf16])
        lh = (C.c_void_p * m)(*[int(a) for a in d_layouts])
        nh = np.ascontiguousarray(n_rows, dtype=np.int64)
        hist = np.zeros(max(1, p.steps), dtype=np.float32)
        self._ctx._check(self._ctx.lib.evoc_mlp_fit_device(
            self.handle, m, xh, lh, _ptr(nh), C.byref(p), _ptr(hist)))
        return hist[:p.steps]

    def free(self) -> None:
        if self.handle and self._ctx.handle:  # a closed context freed it already
            self._ctx.lib.evoc_mlp_free(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def default_n_parts(n: int) -> int:
    """label_propagation_init's part count (label_prop.rs:547-549)."""
    return min(max(int(8.0 * np.sqrt(n)), 256), 16384, n)


def procrustes(m, lib_path: str | None = None) -> np.ndarray:
    """evoc_procrustes: the orthogonal R maximising trace(R^T M) (host only)."""
    lib = load_library(lib_path)
    mm = np.ascontiguousarray(m, dtype=np.float64)
    d = mm.shape[0]
    r = np.zeros((d, d), dtype=np.float64)
    rc = lib.evoc_procrustes(_ptr(mm), d, _ptr(r))
    if rc != EVOC_OK:
        raise EvocError(rc, lib.evoc_last_error(None).decode())
    return r


class Context:
    """One CUDA device and stream (evoc_ctx_t)."""

    def __init__(self, device: int = 0, lib_path: str | None = None):
        self.lib = load_library(lib_path)
        self._children = weakref.WeakSet()  # live graphs and plans, freed by close()
        h = C.c_void_p()
        rc = self.lib.evoc_ctx_create(device, C.byref(h))
        if rc != EVOC_OK:
            raise EvocError(rc, self.lib.evoc_last_error(None).decode())
        self.handle = h

    def mlp(self, in_dim: int, hidden: int, out_dim: int, seed: int = 0) -> Mlp:
        h = C.c_void_p()
        self._check(self.lib.evoc_mlp_create(self.handle, in_dim, hidden, out_dim, seed,
                                             C.byref(h)))
        return Mlp(self, h, in_dim, hidden, out_dim)

    def to_bf16_device(self, d_in: int, count: int, d_out: int) -> None:
        self._check(self.lib.evoc_to_bf16_device(self.handle, C.c_void_p(d_in), int(count),
                                                 C.c_void_p(d_out)))

    def gather_peak(self, nbytes: int = 64 << 20) -> float:
        """Measured L2 random-gather GB/s for 32-byte rows over an nbytes buffer."""
        g = C.c_double()
        self._check(self.lib.evoc_gather_peak(self.handle, int(nbytes), C.byref(g)))
        return g.value

    def smooth_knn_steps(self) -> int:
        """Row-sum evaluations (bisection steps over all rows) of the most
        recent smooth_knn_dist pass on this context."""
        v = C.c_int64()
        self._check(self.lib.evoc_ctx_smooth_knn_steps(self.handle, C.byref(v)))
        return v.value

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return self.lib.evoc_ctx_stream(self.handle) or 0

    def _check(self, rc: int) -> None:
        if rc != EVOC_OK:
            raise EvocError(rc, self.lib.evoc_last_error(self.handle).decode())

    def close(self) -> None:
        """Frees the context's live graphs and plans, then the context."""
        if getattr(self, "handle", None):
            for child in list(self._children):
                child.free()
            self.lib.evoc_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- fuzzy simplicial set -------------------------------------------
    def smooth_knn_dist(self, dists, k: int, local_connectivity: float = 1.0,
                        n_iter: int = 64, row_len=None):
        d = _f32(dists)
        n, kk = d.shape
        rl = None if row_len is None else np.ascontiguousarray(row_len, dtype=np.int32)
        sig = np.zeros(n, dtype=np.float32)
        rho = np.zeros(n, dtype=np.float32)
        self._check(self.lib.evoc_smooth_knn_dist(self.handle, _ptr(d), _ptr(rl), n, kk, int(k),
                                                  float(local_connectivity), int(n_iter),
                                                  _ptr(sig), _ptr(rho)))
        return sig, rho

    def fuzzy_set(self, knn_idx, knn_dist, effective_n_neighbours: float,
                  symmetrise: bool = True) -> Graph:
        idx = np.ascontiguousarray(knn_idx, dtype=np.uint32)
        dist = _f32(knn_dist)
        if idx.ndim != 2 or idx.shape != dist.shape:
            raise EvocError(EVOC_ERR_INVALID_ARGUMENT, "knn_idx/knn_dist must be n x k")
        h = C.c_void_p()
        self._check(self.lib.evoc_fuzzy_set(self.handle, _ptr(idx), _ptr(dist), idx.shape[0],
                                            idx.shape[1], float(effective_n_neighbours),
                                            int(bool(symmetrise)), C.byref(h)))
        return Graph(self, h)

    def fuzzy_set_device(self, d_idx: int, d_dist: int, n: int, k: int,
                         effective_n_neighbours: float, symmetrise: bool = True,
                         d_sigmas: int | None = None, d_rhos: int | None = None) -> Graph:
        h = C.c_void_p()
        self._check(self.lib.evoc_fuzzy_set_device(
            self.handle, C.c_void_p(d_idx), C.c_void_p(d_dist), n, k,
            float(effective_n_neighbours), int(bool(symmetrise)),
            C.c_void_p(d_sigmas) if d_sigmas else None,
            C.c_void_p(d_rhos) if d_rhos else None, C.byref(h)))
        return Graph(self, h)

    def fuzzy_set_device_raw(self, d_idx_raw: int, d_dist_raw: int, n: int, k_raw: int, k: int,
                             effective_n_neighbours: float, symmetrise: bool = True) -> Graph:
        """Fuzzy set from a raw device kNN result (k_raw candidates per row that may
        include the query): self removed and the first k kept, on the device."""
        h = C.c_void_p()
        self._check(self.lib.evoc_fuzzy_set_device_raw(
            self.handle, C.c_void_p(d_idx_raw), C.c_void_p(d_dist_raw), int(n), int(k_raw),
            int(k), float(effective_n_neighbours), int(bool(symmetrise)), C.byref(h)))
        return Graph(self, h)

    def label_prop_partition(self, graph: Graph, approx_n_parts: int | None = None,
                             n_iter: int = 20, seed: int = 42) -> tuple[np.ndarray, int]:
        """label_prop_loop (label_prop.rs:202-230) on a device graph; the default
        part count is label_propagation_init's clamp(8 sqrt(n), 256, 16384), <= n."""
        n = graph.n
        if approx_n_parts is None:
            approx_n_parts = default_n_parts(n)
        part = np.zeros(n, dtype=np.uint32)
        k = C.c_int64()
        self._check(self.lib.evoc_label_prop_partition(self.handle, graph.handle,
                                                       int(approx_n_parts), int(n_iter),
                                                       int(seed), _ptr(part), C.byref(k)))
        return part, k.value

    def label_propagation_init(self, graph: Graph, dim: int, data=None,
                               seed: int = 42) -> np.ndarray:
        """label_propagation_init (label_prop.rs:537-564): the n x dim initial
        embedding of evoc(); data (n x d f32) feeds the PCA base case."""
        n = graph.n
        out = np.zeros((n, dim), dtype=np.float32)
        x = None if data is None else _f32(data)
        d = 0 if x is None else x.shape[1]
        self._check(self.lib.evoc_label_propagation_init(self.handle, graph.handle, int(dim),
                                                         _ptr(x), int(d), int(seed), _ptr(out)))
        return out

    def label_propagation_init_device(self, graph: Graph, dim: int, d_data: int | None,
                                      d: int, seed: int, d_out: int) -> None:
        self._check(self.lib.evoc_label_propagation_init_device(
            self.handle, graph.handle, int(dim), C.c_void_p(d_data) if d_data else None, int(d),
            int(seed), C.c_void_p(d_out)))

    def build_mst(self, data, min_samples: int = 5):
        """build_mst (src/clustering/mst.rs:82-166): the minimum spanning tree
        over mutual reachability of the rows of data (n x dim f32), as
        (u, v, weight) arrays of its edges in insertion order."""
        x = _f32(data)
        if x.ndim != 2:
            raise EvocError(EVOC_ERR_INVALID_ARGUMENT, "data must be n x dim")
        n, dim = x.shape
        m = max(n - 1, 0)
        u = np.zeros(max(m, 1), np.int64)
        v = np.zeros(max(m, 1), np.int64)
        w = np.zeros(max(m, 1), np.float32)
        ne = C.c_int64()
        self._check(self.lib.evoc_build_mst(self.handle, _ptr(x), int(n), int(dim),
                                            int(min_samples), _ptr(u), _ptr(v), _ptr(w),
                                            C.byref(ne)))
        k = ne.value
        return u[:k], v[:k], w[:k]

    def build_mst_device(self, d_data: int, n: int, dim: int, min_samples: int, d_u: int,
                         d_v: int, d_w: int) -> int:
        """build_mst of device points into device outputs; returns the edge count."""
        ne = C.c_int64()
        self._check(self.lib.evoc_build_mst_device(
            self.handle, C.c_void_p(d_data), int(n), int(dim), int(min_samples),
            C.c_void_p(d_u), C.c_void_p(d_v), C.c_void_p(d_w), C.byref(ne)))
        return ne.value

    def graph_from_csr(self, indptr, indices, weights) -> Graph:
        ip = np.ascontiguousarray(indptr, dtype=np.int64)
        ix = np.ascontiguousarray(indices, dtype=np.uint32)
        w = _f32(weights)
        h = C.c_void_p()
        self._check(self.lib.evoc_graph_from_csr(self.handle, _ptr(ip), _ptr(ix), _ptr(w),
                                                 len(ip) - 1, C.byref(h)))
        return Graph(self, h)

    def graph_from_adjacency(self, adj: Sequence[Sequence[tuple[int, float]]]) -> Graph:
        """Upload a Vec<Vec<(usize, T)>>-style adjacency list."""
        indptr = np.zeros(len(adj) + 1, dtype=np.int64)
        for i, row in enumerate(adj):
            indptr[i + 1] = indptr[i] + len(row)
        indices = np.array([j for row in adj for j, _ in row], dtype=np.uint32)
        weights = np.array([w for row in adj for _, w in row], dtype=np.float32)
        return self.graph_from_csr(indptr, indices, weights)

    # ---- embedding ------------------------------------------------------
    def embed(self, graph: Graph, dim: int, params: EvocEmbeddingParams | None = None,
              init=None, seed: int = 42, verbose: int = 0,
              out: np.ndarray | None = None) -> np.ndarray:
        p = (params or EvocEmbeddingParams()).to_c()
        n = graph.n
        if out is None:
            out = np.zeros((n, dim), dtype=np.float32)
        elif out.shape != (n, dim) or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise EvocError(EVOC_ERR_INVALID_ARGUMENT, "out must be a contiguous f32 n x dim array")
        ini = None if init is None else _f32(init)
        if ini is not None and ini.shape != (n, dim):
            raise EvocError(EVOC_ERR_INVALID_ARGUMENT, "init must be n x dim")
        self._check(self.lib.evoc_embed(self.handle, graph.handle, dim, C.byref(p), _ptr(ini),
                                        C.c_uint64(seed), verbose, _ptr(out)))
        return out

    def plan(self, graph: Graph, dim: int, params: EvocEmbeddingParams | None = None,
             seed: int = 42) -> Plan:
        pr = params or EvocEmbeddingParams()
        p = pr.to_c()
        h = C.c_void_p()
        self._check(self.lib.evoc_plan_create(self.handle, graph.handle, dim, C.byref(p),
                                              C.c_uint64(seed), C.byref(h)))
        return Plan(self, h, graph.n, dim, pr.n_epochs)

    def plan_batched(self, graphs: Sequence[Graph], dim: int,
                     params: EvocEmbeddingParams | None = None,
                     seeds: Sequence[int] | None = None) -> Plan:
        """One plan over many graphs; its device rows are the problems' rows in order."""
        pr = params or EvocEmbeddingParams()
        p = pr.to_c()
        m = len(graphs)
        gh = (C.c_void_p * m)(*[g.handle for g in graphs])
        sd = (C.c_uint64 * m)(*(seeds if seeds is not None else [42] * m))
        h = C.c_void_p()
        self._check(self.lib.evoc_plan_create_batched(self.handle, m, gh, dim, C.byref(p), sd,
                                                      C.byref(h)))
        return Plan(self, h, sum(g.n for g in graphs), dim, pr.n_epochs)

    def fuzzy_set_batched(self, knn: Sequence[tuple[np.ndarray, np.ndarray]],
                          effective_n_neighbours: float, symmetrise: bool = True) -> Graph:
        """One block-diagonal graph from many problems' (idx, dist) kNN lists."""
        m = len(knn)
        idx = [np.ascontiguousarray(i, dtype=np.uint32) for i, _ in knn]
        dst = [_f32(d) for _, d in knn]
        k = idx[0].shape[1]
        if any(i.ndim != 2 or i.shape[1] != k or i.shape != d.shape for i, d in zip(idx, dst)):
            raise EvocError(EVOC_ERR_INVALID_ARGUMENT, "every problem needs n x k arrays")
        ih = (C.c_void_p * m)(*[i.ctypes.data for i in idx])
        dh = (C.c_void_p * m)(*[d.ctypes.data for d in dst])
        nh = (C.c_int64 * m)(*[i.shape[0] for i in idx])
        h = C.c_void_p()
        self._check(self.lib.evoc_fuzzy_set_batched(self.handle, m, ih, dh, nh, k,
                                                    float(effective_n_neighbours),
                                                    int(bool(symmetrise)), C.byref(h)))
        return Graph(self, h)

    def plan_blocks(self, graph: Graph, sizes: Sequence[int], dim: int,
                    params: EvocEmbeddingParams | None = None,
                    seeds: Sequence[int] | None = None) -> Plan:
        """A plan over the blocks of a block-diagonal graph (block q: sizes[q] rows)."""
        pr = params or EvocEmbeddingParams()
        p = pr.to_c()
        m = len(sizes)
        nh = (C.c_int64 * m)(*sizes)
        sd = (C.c_uint64 * m)(*(seeds if seeds is not None else [42] * m))
        h = C.c_void_p()
        self._check(self.lib.evoc_plan_create_blocks(self.handle, graph.handle, m, nh, dim,
                                                     C.byref(p), sd, C.byref(h)))
        return Plan(self, h, int(sum(sizes)), dim, pr.n_epochs)

    def embed_blocks(self, graph: Graph, sizes: Sequence[int], dim: int,
                     params: EvocEmbeddingParams | None = None,
                     inits: Sequence[np.ndarray] | None = None,
                     seeds: Sequence[int] | None = None) -> list[np.ndarray]:
        """Embeddings of the blocks of a block-diagonal graph, one array per block."""
        p = (params or EvocEmbeddingParams()).to_c()
        m = len(sizes)
        outs = [np.zeros((n, dim), dtype=np.float32) for n in sizes]
        nh = (C.c_int64 * m)(*sizes)
        oh = (C.c_void_p * m)(*[o.ctypes.data for o in outs])
        sd = (C.c_uint64 * m)(*(seeds if seeds is not None else [42] * m))
        keep = None
        ih = None
        if inits is not None:
            keep = [_f32(x) for x in inits]
            ih = (C.c_void_p * m)(*[x.ctypes.data for x in keep])
        self._check(self.lib.evoc_embed_blocks(self.handle, graph.handle, m, nh, dim,
                                               C.byref(p), ih, sd, oh))
        return outs

    def embed_batched(self, graphs: Sequence[Graph], dim: int,
                      params: EvocEmbeddingParams | None = None,
                      inits: Sequence[np.ndarray] | None = None,
                      seeds: Sequence[int] | None = None) -> list[np.ndarray]:
        p = (params or EvocEmbeddingParams()).to_c()
        m = len(graphs)
        outs = [np.zeros((g.n, dim), dtype=np.float32) for g in graphs]
        gh = (C.c_void_p * m)(*[g.handle for g in graphs])
        oh = (C.c_void_p * m)(*[o.ctypes.data for o in outs])
        sd = (C.c_uint64 * m)(*(seeds if seeds is not None else [42] * m))
        keep = None
        ih = None
        if inits is not None:
            keep = [_f32(x) for x in inits]
            ih = (C.c_void_p * m)(*[x.ctypes.data for x in keep])
        self._check(self.lib.evoc_embed_batched(self.handle, m, gh, dim, C.byref(p), ih, sd, oh))
        return outs


# ---- reference-named functions -----------------------------------------------
def build_fuzzy_simplicial_set(ctx: Context, knn_indices, knn_dists,
                               effective_n_neighbours: float, symmetrise: bool) -> Graph:
    """build_fuzzy_simplicial_set (fuzzy_graph.rs:275-295); the graph stays on the GPU."""
    return ctx.fuzzy_set(knn_indices, knn_dists, effective_n_neighbours, symmetrise)


def coo_to_adjacency_list(graph: Graph) -> list[list[tuple[int, float]]]:
    """coo_to_adjacency_list (fuzzy_graph.rs:242-256) of a device graph, on the host."""
    indptr, indices, weights = graph.export()
    return [[(int(indices[p]), float(weights[p])) for p in range(indptr[i], indptr[i + 1])]
            for i in range(len(indptr) - 1)]


def evoc_embedding(ctx: Context, graph: Graph, n_components: int,
                   params: EvocEmbeddingParams | None = None, initial_embedding=None,
                   seed: int = 42, verbose: int = 0) -> np.ndarray:
    """evoc_embedding (embedding.rs:48-298)."""
    return ctx.embed(graph, n_components, params, initial_embedding, seed, verbose)
