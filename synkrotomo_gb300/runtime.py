"""Host runtime over libsynk: contexts bound to torch's CUDA streams, argument
conversion and checks in the reference's terms, and the device-array object
returned by the drop-in entry points.

PyTorch is used for device memory and streams only; every computation is a
libsynk kernel.
"""
from __future__ import annotations

import ctypes
import math
import threading

import numpy as np
import torch

from . import _lib

__all__ = [
    "SynkError", "DeviceArray", "context", "to_device_f32", "forwardprojection", "backprojection", "sirt",
    "sirt_slices", "sirt3d",
]


class SynkError(RuntimeError):
    """A libsynk call failed; ``code`` is the SYNK_* status."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class _Context:
    def __init__(self, device: int):
        L = _lib.load()
        h = ctypes.c_void_p()
        rc = L.synk_context_new(ctypes.byref(h), int(device), None)
        if rc != 0:
            raise SynkError(rc, f"synk_context_new(device={device}) failed with status {rc}")
        self.handle = h
        self.device = int(device)
        self.lib = L

    def bind(self, stream: torch.cuda.Stream | None = None):
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        self.lib.synk_context_set_stream(self.handle, ctypes.c_void_p(st.cuda_stream))
        return self

    def check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.synk_context_get_error(self.handle).decode()
            if rc == _lib.SYNK_EINVAL:
                raise ValueError(f"{what}: {msg}")
            raise SynkError(rc, f"{what}: {msg}")

    def sync(self):
        rc = self.lib.synk_context_sync(self.handle)
        self.check(rc, "synk_context_sync")

    def set_barrier_limit(self, timeout_ns: int = 2_000_000_000, missing_blocks: int = 0):
        """Time limit of the persistent kernels' waits; ``missing_blocks`` > 0
        injects a barrier that waits for blocks that never arrive (testing
        the SYNK_ETIMEOUT path; 0 in production)."""
        self.check(self.lib.synk_context_set_barrier_limit(self.handle, int(timeout_ns), int(missing_blocks)),
                   "synk_context_set_barrier_limit")


_contexts: dict[int, _Context] = {}
_ctx_lock = threading.Lock()


def context(device: int | None = None) -> _Context:
    """The libsynk context of ``device`` (default: torch's current device),
    bound to torch's current stream on that device."""
    if not torch.cuda.is_available():
        raise RuntimeError("synkrotomo_gb300 needs a CUDA GPU (no CPU fallback exists)")
    dev = torch.cuda.current_device() if device is None else int(device)
    with _ctx_lock:
        ctx = _contexts.get(dev)
        if ctx is None:
            ctx = _contexts[dev] = _Context(dev)
    return ctx.bind()


def _ptr(t: torch.Tensor | None):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


# ---------------------------------------------------------------------------
# argument conversion, in the reference's terms
# ---------------------------------------------------------------------------

def to_device_f32(x, argno: int, name: str, device=None) -> torch.Tensor:
    """A contiguous 1-D float32 CUDA tensor holding ``x``.

    Like the reference's generated entry points, arrays must already be
    float32; anything else raises TypeError (there is no silent cast).
    Multi-dimensional inputs are flattened (the reference takes flattened
    arrays, README.md:24).
    """
    if isinstance(x, torch.Tensor):
        if x.dtype != torch.float32:
            raise TypeError(f"Argument #{argno} ({name}) has invalid value\nFuthark type: []f32\n"
                            f"Argument has torch dtype {x.dtype}")
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        return x.reshape(-1).to(dev, non_blocking=True).contiguous()
    if hasattr(x, "get") and not isinstance(x, np.ndarray):      # DeviceArray or a pyopencl-like array
        if isinstance(x, DeviceArray):
            return to_device_f32(x.torch(), argno, name, device)
        x = x.get()
    arr = np.asarray(x)
    if arr.dtype != np.float32:
        raise TypeError(f"Argument #{argno} ({name}) has invalid value\nFuthark type: []f32\n"
                        f"Argument has Python type {type(x).__name__} and dtype {arr.dtype}")
    t = torch.from_numpy(np.ascontiguousarray(arr.reshape(-1)))
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    if t.numel() and not t.is_pinned():
        return t.to(dev)
    return t.to(dev, non_blocking=True)


def scalar_f32(v, argno: int, name: str) -> float:
    try:
        f = np.float32(v)
    except (TypeError, ValueError):
        raise TypeError(f"Argument #{argno} ({name}) has invalid value\nFuthark type: f32\n"
                        f"Argument has Python type {type(v).__name__} and value: {v!r}") from None
    if isinstance(v, (np.ndarray,)) and np.ndim(v) != 0:
        raise TypeError(f"Argument #{argno} ({name}) must be a scalar f32")
    return float(f)


def scalar_i32(v, argno: int, name: str) -> int:
    if isinstance(v, (bool, np.bool_)) or not isinstance(v, (int, np.integer)):
        if isinstance(v, (float, np.floating)) and float(v).is_integer():
            v = int(v)
        else:
            raise TypeError(f"Argument #{argno} ({name}) has invalid value\nFuthark type: i32\n"
                            f"Argument has Python type {type(v).__name__} and value: {v!r}")
    iv = int(v)
    if not (-2 ** 31 <= iv < 2 ** 31):
        raise TypeError(f"Argument #{argno} ({name}) does not fit in i32: {iv}")
    return iv


class DeviceArray:
    """Result of an entry point: a flattened float32 device array.

    ``get()`` copies it to a NumPy array (as ``pyopencl.array.Array.get()``
    does for the reference's generated classes) after checking that the
    kernels that produced it completed without error.
    """

    def __init__(self, tensor: torch.Tensor, ctx: _Context):
        self._t = tensor
        self._ctx = ctx

    def torch(self) -> torch.Tensor:
        return self._t

    def get(self) -> np.ndarray:
        self._ctx.sync()
        return self._t.detach().cpu().numpy()

    @property
    def shape(self):
        return tuple(self._t.shape)

    @property
    def dtype(self):
        return np.dtype(np.float32)

    def __len__(self):
        return self._t.numel()

    def __array__(self, dtype=None, copy=None):
        a = self.get()
        return a if dtype is None else a.astype(dtype)

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, dtype=float32, device={self._t.device})"


# ---------------------------------------------------------------------------
# operations on device tensors
# ---------------------------------------------------------------------------

def forwardprojection(angles: torch.Tensor, rhozero: float, deltarho: float, numrhos: int, image: torch.Tensor,
                      out: torch.Tensor | None = None, sparse: bool = False) -> torch.Tensor:
    """Angle-major sinogram [a*numrhos] of ``image`` (futhark/forwardprojection.fut:71-84)."""
    ctx = context(image.device.index)
    a = angles.numel()
    if out is None:
        out = torch.empty(a * int(numrhos), dtype=torch.float32, device=image.device)
    fn = ctx.lib.synk_forwardprojection_sparse if sparse else ctx.lib.synk_forwardprojection
    rc = fn(ctx.handle, _ptr(out), _ptr(angles), a, rhozero, deltarho, int(numrhos), _ptr(image), image.numel())
    ctx.check(rc, "forwardprojection")
    return out


def backprojection(angles: torch.Tensor, rhozero: float, deltarho: float, size: int, projections: torch.Tensor,
                   out: torch.Tensor | None = None, sparse: bool = False) -> torch.Tensor:
    """Image [size*size] backprojected from ``projections`` (futhark/backprojection.fut:82-93)."""
    ctx = context(projections.device.index)
    a = angles.numel()
    side = (int(size) // 2) * 2
    if out is None:
        out = torch.empty(side * side, dtype=torch.float32, device=projections.device)
    fn = ctx.lib.synk_backprojection_sparse if sparse else ctx.lib.synk_backprojection
    rc = fn(ctx.handle, _ptr(out), _ptr(angles), a, rhozero, deltarho, int(size), _ptr(projections),
            projections.numel())
    ctx.check(rc, "backprojection")
    return out


def sirt_slices(angles: torch.Tensor, rhozero: float, deltarho: float, numrhos: int, size: int, nslices: int,
                image: torch.Tensor | None, projections: torch.Tensor, iterations: int, tol: float = 0.0,
                residuals: bool = False, fp_split: int = 0, bp_split: int = 0, grid_blocks: int = 0,
                out: torch.Tensor | None = None):
    """SIRT of ``nslices`` independent slices in one persistent launch.

    Returns ``(x, res, done)``: x [nslices*size*size]; res [nslices,
    iterations+1] relative residuals ||FP(x_k)-b||/||b|| (float64, None unless
    ``residuals``); done [nslices] number of updates applied (int32).
    """
    ctx = context(projections.device.index)
    dev = projections.device
    n = int(size) * int(size)
    if out is None:
        out = torch.empty(int(nslices) * n, dtype=torch.float32, device=dev)
    res = None
    if residuals:
        res = torch.full((int(nslices), int(iterations) + 1), float("nan"), dtype=torch.float64, device=dev)
    done = torch.zeros(int(nslices), dtype=torch.int32, device=dev)
    opts = _lib.SynkOptions(float(tol), res.data_ptr() if res is not None else None, done.data_ptr(),
                            int(fp_split), int(bp_split), int(grid_blocks))
    rc = ctx.lib.synk_sirt_slices(ctx.handle, _ptr(out), _ptr(angles), angles.numel(), rhozero, deltarho,
                                  int(numrhos), int(size), int(nslices), _ptr(image), _ptr(projections),
                                  int(iterations), ctypes.byref(opts))
    ctx.check(rc, "sirt")
    return out, res, done


class Problem:
    """One problem of a batched SIRT launch (a stack of slices with one geometry)."""

    def __init__(self, angles: torch.Tensor, rhozero: float, deltarho: float, numrhos: int, size: int,
                 projections: torch.Tensor, iterations: int, nslices: int = 1, image: torch.Tensor | None = None,
                 residuals: bool = False, fp_split: int = 0, bp_split: int = 0):
        self.angles, self.rhozero, self.deltarho = angles, float(rhozero), float(deltarho)
        self.numrhos, self.size, self.nslices = int(numrhos), int(size), int(nslices)
        self.projections, self.iterations, self.image = projections, int(iterations), image
        self.fp_split, self.bp_split = int(fp_split), int(bp_split)
        dev = projections.device
        self.out = torch.empty(self.nslices * self.size * self.size, dtype=torch.float32, device=dev)
        self.residuals = (torch.full((self.nslices, self.iterations + 1), float("nan"), dtype=torch.float64,
                                     device=dev) if residuals else None)
        self.done = torch.zeros(self.nslices, dtype=torch.int32, device=dev)

    def _desc(self):
        return _lib.SynkProblem(self.angles.data_ptr(), self.angles.numel(), self.rhozero, self.deltarho,
                                self.numrhos, self.size, self.nslices, self.iterations,
                                self.image.data_ptr() if self.image is not None else None,
                                self.projections.data_ptr(), self.out.data_ptr(),
                                self.residuals.data_ptr() if self.residuals is not None else None,
                                self.done.data_ptr(), self.fp_split, self.bp_split)


def resident_blocks() -> int:
    """Blocks of the persistent SIRT kernel that fit on the device at once:
    ``grid_blocks`` of that value forces the persistent engine with its full
    grid, -1 the phase-split engine, 0 lets the library choose."""
    context()
    return int(_lib.load().synk_sirt_resident_blocks())


def sirt_batch(problems: list, tol: float = 0.0, grid_blocks: int = 0) -> list:
    """Every problem's SIRT in one persistent launch (``synk_sirt_batch``);
    results land in each problem's ``out`` / ``residuals`` / ``done``."""
    if not problems:
        return problems
    ctx = context(problems[0].projections.device.index)
    arr = (_lib.SynkProblem * len(problems))(*[p._desc() for p in problems])
    rc = ctx.lib.synk_sirt_batch(ctx.handle, len(problems), arr, float(tol), int(grid_blocks))
    ctx.check(rc, "sirt_batch")
    return problems


class SirtPlan:
    """A batched SIRT solve captured in a CUDA graph (``synk_sirt_plan_*``).

    The problems' tensors are bound at creation; refill them in place and call
    ``launch()`` to solve again."""

    def __init__(self, problems: list, tol: float = 0.0, grid_blocks: int = 0):
        self.problems = problems
        self.ctx = context(problems[0].projections.device.index)
        arr = (_lib.SynkProblem * len(problems))(*[p._desc() for p in problems])
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.synk_sirt_plan_new(self.ctx.handle, ctypes.byref(h), len(problems), arr,
                                                       float(tol), int(grid_blocks)), "synk_sirt_plan_new")
        self._h = h

    def launch(self):
        ctx = context(self.ctx.device)
        ctx.check(ctx.lib.synk_sirt_plan_launch(ctx.handle, self._h), "synk_sirt_plan_launch")
        return self.problems

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self.ctx.lib.synk_sirt_plan_free(h)
            except Exception:
                pass
            self._h = None


def sirt(angles: torch.Tensor, rhozero: float, deltarho: float, image: torch.Tensor, projections: torch.Tensor,
         iterations: int, out: torch.Tensor | None = None) -> torch.Tensor:
    """``iterations`` SIRT updates from ``image`` (futhark/SIRT.fut:43-49)."""
    ctx = context(projections.device.index)
    if out is None:
        out = torch.empty(image.numel(), dtype=torch.float32, device=projections.device)
    rc = ctx.lib.synk_SIRT(ctx.handle, _ptr(out), _ptr(angles), angles.numel(), rhozero, deltarho, _ptr(image),
                           image.numel(), _ptr(projections), projections.numel(), int(iterations))
    ctx.check(rc, "SIRT")
    return out


def sirt3d(angles: torch.Tensor, rhos: torch.Tensor, projections: torch.Tensor, iterations: int, size: int,
           out: torch.Tensor | None = None, nslices: int | None = None) -> torch.Tensor:
    """``size`` slices reconstructed independently (futhark/SIRT3D.fut:18-29),
    with rhozero = rhos[0] and deltarho = rhos[1] - rhos[0] (float32).

    ``nslices``: a stack of that many ``size`` x ``size`` slices instead of
    ``size`` (projections then hold nslices*a*len(rhos) values)."""
    if nslices is not None:
        ns, r = int(nslices), rhos.numel()
        if ns < 1:
            raise ValueError(f"nslices must be positive (got {ns})")
        if r < 2:
            raise ValueError(f"rhos needs at least two detector positions (got {r})")
        if projections.numel() != ns * angles.numel() * r:
            raise ValueError(f"projections has {projections.numel()} values, expected nslices*a*r = "
                             f"{ns * angles.numel() * r}")
        rh = rhos[:2].detach().cpu().numpy().astype(np.float32)
        deltarho = float(np.float32(rh[1]) - np.float32(rh[0]))
        x, _, _ = sirt_slices(angles, float(rh[0]), deltarho, r, size, ns, None, projections, iterations, out=out)
        return x
    ctx = context(projections.device.index)
    if out is None:
        out = torch.empty(int(size) ** 3, dtype=torch.float32, device=projections.device)
    rc = ctx.lib.synk_SIRT3D(ctx.handle, _ptr(out), _ptr(angles), angles.numel(), _ptr(rhos), rhos.numel(),
                             _ptr(projections), projections.numel(), int(iterations), int(size))
    ctx.check(rc, "SIRT3D")
    return out


def compare(sane: torch.Tensor, test: torch.Tensor, tol: float = 0.05) -> tuple:
    """(count, sse, all_ok) of futhark/tools/{diff,mse,sanityCheck}.fut in one
    pass: the indices i > 0 with |sane-test| > tol, the FP64 sum of squared
    differences, and whether every |sane-test| < tol."""
    if sane.numel() != test.numel():
        raise ValueError(f"compare: lengths differ ({sane.numel()} vs {test.numel()})")
    ctx = context(sane.device.index)
    res = torch.empty(3, dtype=torch.float64, device=sane.device)   # 24 B: synk_compare_result
    rc = ctx.lib.synk_compare(ctx.handle, _ptr(res), _ptr(sane), _ptr(test), sane.numel(), float(tol))
    ctx.check(rc, "compare")
    raw = res.cpu().numpy().view(np.uint8)
    count = int(raw[:8].view(np.uint64)[0])
    sse = float(raw[8:16].view(np.float64)[0])
    ok = bool(raw[16:20].view(np.int32)[0])
    return count, sse, ok


def compare_program(name: str, sane: torch.Tensor, test: torch.Tensor):
    """The result of tools/diff.fut (np.int32), mse.fut (np.float32) or
    sanityCheck.fut (np.bool_), computed on the GPU."""
    if sane.numel() != test.numel():
        raise ValueError(f"{name}: lengths differ ({sane.numel()} vs {test.numel()})")
    ctx = context(sane.device.index)
    kind = {"diff": (ctx.lib.synk_diff, torch.int32), "mse": (ctx.lib.synk_mse, torch.float32),
            "sanityCheck": (ctx.lib.synk_sanityCheck, torch.uint8)}
    fn, dt = kind[name]
    out = torch.empty(1, dtype=dt, device=sane.device)
    ctx.check(fn(ctx.handle, _ptr(out), _ptr(sane), _ptr(test), sane.numel()), name)
    v = out.cpu().numpy()[0]
    return np.bool_(v != 0) if name == "sanityCheck" else v


def image_side(n: int) -> int:
    s = math.isqrt(int(n))
    return s


class SystemMatrix:
    """The forward projector's rule as a CSR matrix A (rays x pixels) and its
    exact transpose, built and held on the GPU (``synk_csr_*`` of the C ABI)."""

    def __init__(self, angles: torch.Tensor, rhozero: float, deltarho: float, numrhos: int, size: int):
        self._ctx = context(angles.device.index)
        self.device = angles.device
        h = ctypes.c_void_p()
        rc = self._ctx.lib.synk_csr_new(self._ctx.handle, ctypes.byref(h), _ptr(angles), angles.numel(),
                                        float(rhozero), float(deltarho), int(numrhos), int(size))
        self._ctx.check(rc, "synk_csr_new")
        self._h = h
        r, c, z = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._ctx.lib.synk_csr_shape(h, ctypes.byref(r), ctypes.byref(c), ctypes.byref(z))
        self.rows, self.cols, self.nnz = r.value, c.value, z.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._ctx.lib.synk_csr_free(h)
            except Exception:
                pass
            self._h = None

    def matvec(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        ctx = context(self.device.index)
        if out is None:
            out = torch.empty(self.rows, dtype=torch.float32, device=self.device)
        ctx.check(ctx.lib.synk_csr_spmv(ctx.handle, self._h, _ptr(x), _ptr(out)), "synk_csr_spmv")
        return out

    def rmatvec(self, y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        ctx = context(self.device.index)
        if out is None:
            out = torch.empty(self.cols, dtype=torch.float32, device=self.device)
        ctx.check(ctx.lib.synk_csr_spmv_t(ctx.handle, self._h, _ptr(y), _ptr(out)), "synk_csr_spmv_t")
        return out

    def arrays(self, transpose: bool = False):
        """(rowptr int64, colidx int32, vals float32) of A or A^T as device tensors (views)."""
        p, i, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        self._ctx.lib.synk_csr_arrays(self._h, int(transpose), ctypes.byref(p), ctypes.byref(i), ctypes.byref(v))
        n = self.cols if transpose else self.rows
        return (device_view(p.value, n + 1, "<i8", self.device), device_view(i.value, self.nnz, "<i4", self.device),
                device_view(v.value, self.nnz, "<f4", self.device))


class _CudaArray:
    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def device_view(ptr: int, n: int, typestr: str, device) -> torch.Tensor:
    """A torch tensor viewing ``n`` elements of library-owned device memory."""
    if n == 0:
        dt = {"<i8": torch.int64, "<i4": torch.int32, "<f4": torch.float32}[typestr]
        return torch.empty(0, dtype=dt, device=device)
    return torch.as_tensor(_CudaArray(ptr, n, typestr), device=device)
