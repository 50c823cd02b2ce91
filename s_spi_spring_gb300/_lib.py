"""ctypes binding of the engine's C ABI (``include/spe_engine.h``).

The shared library is built in-tree (``s_spi_spring_gb300/_build/libspe.so``,
see ``build.py``).  Loading fails loudly when it is missing: there is no
CPU fallback for the engine.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libspe.so"
_lock = threading.Lock()
_lib = None

SPE_OK = 0
SPE_OP_HIO, SPE_OP_RAAR, SPE_OP_ER, SPE_OP_SW, SPE_OP_SWA = range(5)
SPE_LOSS_AMPLITUDE, SPE_LOSS_POISSON = 0, 1
SPE_RESAMPLE_PLAIN, SPE_RESAMPLE_EWALD, SPE_RESAMPLE_CUT_EWALD, SPE_RESAMPLE_CUT = 0, 1, 2, 3

# Every symbol the header declares, with (restype, argtypes).
_vp = C.c_void_p
_i = C.c_int
_f = C.c_float
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)


class SpeOp(C.Structure):
    _fields_ = [("kind", C.c_int32), ("iterations", C.c_int32), ("beta", C.c_float),
                ("sigma", C.c_float), ("threshold", C.c_float), ("pixels", C.c_int32)]


class SpeMetrics(C.Structure):
    _fields_ = [("error", C.c_float), ("error_fourier", C.c_float), ("error_real", C.c_float),
                ("reality", C.c_float), ("modulesum", C.c_float), ("complexsum", C.c_float),
                ("symmetry", C.c_float)]


SIGNATURES = {
    "spe_last_error": (C.c_char_p, []),
    "spe_version": (_i, []),
    "spe_side_supported": (_i, [_i, C.POINTER(_i)]),
    "spe_device_count": (_i, [C.POINTER(_i)]),
    "spe_device_info": (_i, [_i, C.c_char_p, _i, C.c_char_p, _i]),
    "spe_prepare_pattern": (_i, [_fp, _i, _i, _i, _i, _fp]),
    "spe_create": (_i, [_i, _i, C.POINTER(_vp)]),
    "spe_destroy": (_i, [_vp]),
    "spe_set_stream": (_i, [_vp, _vp]),
    "spe_get_stream": (_i, [_vp, C.POINTER(_vp)]),
    "spe_set_amplitudes": (_i, [_vp, _fp]),
    "spe_get_amplitudes": (_i, [_vp, _fp]),
    "spe_reserve": (_i, [_vp, _i]),
    "spe_capacity": (_i, [_vp, C.POINTER(_i)]),
    "spe_upload": (_i, [_vp, _i, _i, _fp, _ip]),
    "spe_download": (_i, [_vp, _i, _i, _fp, _ip]),
    "spe_device_buffers": (_i, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    "spe_hio": (_i, [_vp, _i, _i, _i, _f, _f]),
    "spe_raar": (_i, [_vp, _i, _i, _i, _f, _f]),
    "spe_er": (_i, [_vp, _i, _i, _i, _f]),
    "spe_sw": (_i, [_vp, _i, _i, _f, _f, _f]),
    "spe_swa": (_i, [_vp, _i, _i, _f, _i, _f]),
    "spe_evaluate": (_i, [_vp, _i, _i, _f, _f, C.POINTER(SpeMetrics)]),
    "spe_sequence": (_i, [_vp, _i, _i, C.POINTER(SpeOp), _i, _i, _f, _f, C.POINTER(SpeMetrics)]),
    "spe_synchronize": (_i, [_vp]),
    "spe_seed": (_i, [_vp, C.c_uint32]),
    "spe_reshift": (_i, [_vp, _i, _i, _i, _fp, _f, _f]),
    "spe_average": (_i, [_vp, _i, _i, _fp, _f, _i]),
    "spe_average_module": (_i, [_vp, _i, _i, _fp, _i, _f, _fp]),
    "spe_crossover": (_i, [_vp, _i, _i, _fp, _i, _i, _i, _f, _f, _f, _f, _i, _f, _i, _f, _f, _f]),
    "spe_crossover_draws": (_i, [C.c_uint32, _i, _ip, _f, _i, _f, _f, _f, _ip, _fp, _ip, _i, _ip]),
    "spe_set_tiles": (_i, [_vp, _i, _i]),
    "spe_get_tiles": (_i, [_vp, C.POINTER(_i), C.POINTER(_i)]),
    "spe_set_schedule": (_i, [_vp, _i, _i]),
    "spe_get_schedule": (_i, [_vp, C.POINTER(_i), C.POINTER(_i)]),
    "spe_autotune": (_i, [_vp, _i, _i, _i, C.POINTER(_i), C.POINTER(_i)]),
    "spe_iterate_noalloc": (_i, [_i, _vp, _vp, _vp, _i, _i, _i, _f, _f, _vp]),
    "spe_initialize_pop": (_i, [_vp, _i, _i, _i, _f, _f, _i, _i, _f, _f, _f, _f, _f, _f]),
    "spe_copy": (_i, [_vp, _i, _i, _i]),
    "spe_gather": (_i, [_vp, _ip, _i, _i]),
    "spe_iterate_host": (_i, [_vp, _i, _i, _fp, _ip, _i, _i, _f, _f, _fp, _i]),
    "spe_far_field": (_i, [_vp, _i, _i, _fp]),
    "spe_loss_grad": (_i, [_vp, _vp, _vp, _i, _i, _f, _vp, _vp, _vp]),
    "spe_loss_grad_cols": (_i, [_vp, _vp, _vp, _i, _i, _f, _vp, _vp]),
    "spe_selftest_bounded_wait": (_i, [_vp]),
    "spe_grad_rows": (_i, [_vp, _vp, _vp, _i, _vp, _vp]),
    "spe_set_amplitudes_batch": (_i, [_vp, _fp, _i, _i]),
    "spe_adam_step": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _f, _f, _f, _f, _f, _i, _vp]),
    "spe_get_rng_state": (_i, [_vp, C.c_char_p, _i, C.POINTER(_i)]),
    "spe_set_rng_state": (_i, [_vp, C.c_char_p]),
    "spe_pattern_resample": (_i, [_i, _vp, _vp, _i, _i, C.c_double, C.c_double, C.c_double, C.c_double, _i, _i,
                                  _i, _i, _vp, _vp, _i]),
    "spe_pattern_radial_profile": (_i, [_vp, _i, _i, C.c_double, C.c_double, C.c_double, _vp, _i, C.c_double,
                                        C.c_double, _vp, _i]),
    "spe_stream_create": (_i, [C.POINTER(_vp)]),
    "spe_stream_destroy": (_i, [_vp]),
    "spe_graph_begin": (_i, [_vp]),
    "spe_graph_end": (_i, [_vp, C.POINTER(_vp)]),
    "spe_graph_launch": (_i, [_vp, _vp]),
    "spe_graph_destroy": (_i, [_vp]),
}


def stream_create() -> int:
    """A non-blocking CUDA stream (handle) on the current device."""
    st = _vp()
    call("spe_stream_create", C.byref(st))
    return st.value


def stream_destroy(handle: int):
    call("spe_stream_destroy", _vp(handle))


class Graph:
    """A CUDA graph of engine calls recorded on `stream` (a CUDA stream
    handle): ``with Graph.capture(stream) as g: ...`` then ``g.launch()``."""

    def __init__(self, handle, stream):
        self.h, self.stream = handle, stream

    @classmethod
    def capture(cls, stream):
        return _Capture(stream)

    def launch(self, stream=None):
        call("spe_graph_launch", self.h, _vp(stream if stream is not None else self.stream))

    def close(self):
        if self.h:
            load().spe_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Capture:
    def __init__(self, stream):
        self.stream = stream
        self.graph = None

    def __enter__(self):
        call("spe_graph_begin", _vp(self.stream))
        return self

    def __exit__(self, exc_type, exc, tb):
        lib = load()
        g = _vp()
        rc = lib.spe_graph_end(_vp(self.stream), C.byref(g))
        if exc_type is None:
            if rc != SPE_OK:
                raise EngineError("spe_graph_end", rc, lib.spe_last_error().decode())
            self.graph = Graph(g.value, self.stream)
        elif rc == SPE_OK:
            lib.spe_graph_destroy(g)
        return False


class EngineError(RuntimeError):
    """A C ABI call returned a non-zero status."""

    def __init__(self, fn, code, msg):
        super().__init__(f"{fn} failed ({code}): {msg}")
        self.code = code


def library_path() -> Path:
    return _LIB_PATH


def load():
    """Load (once) and return the engine library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _LIB_PATH.exists():
            raise ImportError(
                f"engine library {_LIB_PATH} is not built; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first")
        lib = C.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != SPE_OK:
        raise EngineError(name, rc, lib.spe_last_error().decode())
    return rc


def side_supported(n: int) -> str | None:
    """"compiled" for a side with a compiled plan, "any" for one the any-side
    kernels run, None when the engine rejects it."""
    c = _i(0)
    rc = load().spe_side_supported(int(n), C.byref(c))
    if rc != SPE_OK:
        return None
    return "compiled" if c.value else "any"


def device_count() -> int:
    """CUDA devices visible to the process (0 without any)."""
    n = _i(0)
    call("spe_device_count", C.byref(n))
    return int(n.value)


def device_info(device: int) -> tuple[str, str]:
    """(name, PCI bus id) of a CUDA device."""
    name = C.create_string_buffer(256)
    bus = C.create_string_buffer(64)
    call("spe_device_info", int(device), name, 256, bus, 64)
    return name.value.decode(), bus.value.decode()


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_fp) if a is not None else None


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip) if a is not None else None


class Engine:
    """Owning handle of one engine (one pattern size, one device)."""

    def __init__(self, n: int, device: int = 0):
        h = _vp()
        call("spe_create", int(n), int(device), C.byref(h))
        self.h = h
        self.n = int(n)
        self.device = int(device)

    def close(self):
        if getattr(self, "h", None):
            load().spe_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- pattern / population ------------------------------------------------
    def set_amplitudes(self, amp):
        amp = np.ascontiguousarray(amp, dtype=np.float32)
        assert amp.shape == (self.n, self.n)
        call("spe_set_amplitudes", self.h, fptr(amp))

    def set_amplitudes_batch(self, amps, individuals_per_pattern):
        """amps: (npatterns, n, n); slot p uses pattern p // individuals_per_pattern."""
        amps = np.ascontiguousarray(amps, dtype=np.float32)
        assert amps.ndim == 3 and amps.shape[1:] == (self.n, self.n)
        call("spe_set_amplitudes_batch", self.h, fptr(amps), int(amps.shape[0]), int(individuals_per_pattern))

    def get_amplitudes(self):
        out = np.empty((self.n, self.n), np.float32)
        call("spe_get_amplitudes", self.h, fptr(out))
        return out

    def reserve(self, capacity: int):
        call("spe_reserve", self.h, int(capacity))

    @property
    def capacity(self) -> int:
        c = C.c_int()
        call("spe_capacity", self.h, C.byref(c))
        return c.value

    def upload(self, first, density=None, support=None):
        d = None if density is None else np.ascontiguousarray(density, dtype=np.complex64)
        s = None if support is None else np.ascontiguousarray(support, dtype=np.int32)
        arr = d if d is not None else s
        count = arr.size // (self.n * self.n)
        self.reserve(first + count)
        call("spe_upload", self.h, int(first), int(count),
             None if d is None else d.view(np.float32).ctypes.data_as(_fp), iptr(s))

    def download(self, first, count, density=True, support=True):
        d = np.empty((count, self.n, self.n), np.complex64) if density else None
        s = np.empty((count, self.n, self.n), np.int32) if support else None
        call("spe_download", self.h, int(first), int(count),
             None if d is None else d.view(np.float32).ctypes.data_as(_fp), iptr(s))
        return d, s

    def set_stream(self, stream_handle: int | None):
        call("spe_set_stream", self.h, _vp(stream_handle or 0))

    def get_stream(self) -> int:
        st = _vp()
        call("spe_get_stream", self.h, C.byref(st))
        return st.value or 0

    def device_buffers(self):
        d, s = _vp(), _vp()
        call("spe_device_buffers", self.h, C.byref(d), C.byref(s))
        return d.value, s.value

    # -- algorithms ------------------------------------------------------------
    def hio(self, first, count, iterations, beta, reality=0.0):
        call("spe_hio", self.h, int(first), int(count), int(iterations), float(beta), float(reality))

    def raar(self, first, count, iterations, beta, reality=0.0):
        call("spe_raar", self.h, int(first), int(count), int(iterations), float(beta), float(reality))

    def er(self, first, count, iterations, reality=0.0):
        call("spe_er", self.h, int(first), int(count), int(iterations), float(reality))

    def sw(self, first, count, sigma, threshold, reality=0.0):
        call("spe_sw", self.h, int(first), int(count), float(sigma), float(threshold), float(reality))

    def swa(self, first, count, sigma, pixels, reality=0.0):
        call("spe_swa", self.h, int(first), int(count), float(sigma), int(pixels), float(reality))

    def evaluate(self, first, count, reality=0.0, realpen=0.0):
        m = (SpeMetrics * max(count, 1))()
        call("spe_evaluate", self.h, int(first), int(count), float(reality), float(realpen), m)
        return [metrics_dict(m[i]) for i in range(count)]

    def sequence(self, first, count, ops, nrep=1, reality=0.0, realpen=0.0, evaluate=True):
        arr = (SpeOp * max(len(ops), 1))(*ops)
        m = (SpeMetrics * max(count, 1))() if evaluate else None
        call("spe_sequence", self.h, int(first), int(count), arr, len(ops), int(nrep),
             float(reality), float(realpen), m)
        return [metrics_dict(m[i]) for i in range(count)] if evaluate else None

    def synchronize(self):
        call("spe_synchronize", self.h)

    # -- tuning ----------------------------------------------------------------
    def set_tiles(self, cols=0, rows=0):
        call("spe_set_tiles", self.h, int(cols), int(rows))

    def tiles(self):
        a, b = C.c_int(), C.c_int()
        call("spe_get_tiles", self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def set_schedule(self, chunk=0, lanes=1):
        call("spe_set_schedule", self.h, int(chunk), int(lanes))

    def schedule(self):
        a, b = C.c_int(), C.c_int()
        call("spe_get_schedule", self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def autotune(self, first, count, iterations=10):
        a, b = C.c_int(), C.c_int()
        call("spe_autotune", self.h, int(first), int(count), int(iterations), C.byref(a), C.byref(b))
        return a.value, b.value

    # -- population-level operations --------------------------------------------
    def rng_state(self) -> str:
        n = C.c_int()
        call("spe_get_rng_state", self.h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value)
        call("spe_get_rng_state", self.h, buf, n.value, C.byref(n))
        return buf.value.decode()

    def set_rng_state(self, state: str):
        call("spe_set_rng_state", self.h, state.encode())

    def seed(self, seed: int):
        call("spe_seed", self.h, C.c_uint32(int(seed) & 0xFFFFFFFF))

    def initialize_pop(self, first, count, support_size, itemsize, nitems=(8, 8), exponent=(0.0, 0.0),
                       scaling=(0.0, 0.0), phaserange=0.0, suppcut=0.0):
        self.reserve(first + count)
        call("spe_initialize_pop", self.h, int(first), int(count), int(support_size), float(itemsize[0]),
             float(itemsize[1]), int(nitems[0]), int(nitems[1]), float(exponent[0]), float(exponent[1]),
             float(scaling[0]), float(scaling[1]), float(phaserange), float(suppcut))

    def copy(self, src, dst, count):
        call("spe_copy", self.h, int(src), int(dst), int(count))

    def loss_grad(self, density_ptr, support_ptr, count, loss=0, eps=0.0, loss_ptr=0, grad_ptr=0, scale_ptr=0):
        """Far-field loss / gradient on device arrays given by address."""
        call("spe_loss_grad", self.h, _vp(density_ptr), _vp(support_ptr), int(count), int(loss), float(eps),
             _vp(loss_ptr or 0), _vp(grad_ptr or 0), _vp(scale_ptr or 0))

    def selftest_bounded_wait(self):
        """Queues the bounded-wait self-test; the next synchronize reports it."""
        call("spe_selftest_bounded_wait", self.h)

    def loss_grad_cols(self, density_ptr, support_ptr, count, half_ptr, loss=0, eps=0.0, loss_ptr=0):
        """Loss and the adjoint up to its column pass, kept in ``half``."""
        call("spe_loss_grad_cols", self.h, _vp(density_ptr), _vp(support_ptr), int(count), int(loss), float(eps),
             _vp(loss_ptr or 0), _vp(half_ptr))

    def grad_rows(self, half_ptr, support_ptr, count, grad_ptr, scale_ptr=0):
        """The adjoint's last pass from ``half`` (grad may be half)."""
        call("spe_grad_rows", self.h, _vp(half_ptr), _vp(support_ptr), int(count), _vp(grad_ptr),
             _vp(scale_ptr or 0))

    def adam_step(self, density_ptr, support_ptr, m_ptr, v_ptr, count, loss=1, eps=0.0, lr=1e-3, beta1=0.9,
                  beta2=0.999, adam_eps=1e-8, step=1, loss_ptr=0):
        """Loss at the current densities, then one fused Adam step in place."""
        call("spe_adam_step", self.h, _vp(density_ptr), _vp(support_ptr), _vp(m_ptr), _vp(v_ptr), int(count),
             int(loss), float(eps), float(lr), float(beta1), float(beta2), float(adam_eps), int(step),
             _vp(loss_ptr or 0))

    def population_arrays(self, first, count):
        """Device addresses of slots [first, first+count): (density, support)."""
        d, s = self.device_buffers()
        off = int(first) * self.n * self.n
        return d + off * 8, s + off * 4

    def iterate_host(self, first, density, support, algorithm, iterations, beta=0.0, reality=0.0, out=None,
                     blocks=0):
        """Host arrays in, iterations, host array out (copies overlapped with
        the iterations of other blocks); returns the densities."""
        d = np.ascontiguousarray(density, dtype=np.complex64)
        s = None if support is None else np.ascontiguousarray(support, dtype=np.int32)
        count = d.size // (self.n * self.n)
        out = np.empty_like(d) if out is None else out
        call("spe_iterate_host", self.h, int(first), int(count), d.view(np.float32).ctypes.data_as(_fp), iptr(s),
             int(algorithm), int(iterations), float(beta), float(reality), out.view(np.float32).ctypes.data_as(_fp),
             int(blocks))
        return out

    def far_field(self, first, count):
        """|FFT+(rho)| of slots [first, first+count), DC at [0, 0]."""
        out = np.empty((count, self.n, self.n), np.float32)
        call("spe_far_field", self.h, int(first), int(count), fptr(out))
        return out

    def gather(self, src_slots, dst_first):
        src = np.ascontiguousarray(src_slots, dtype=np.int32)
        call("spe_gather", self.h, iptr(src), int(src.size), int(dst_first))

    def reshift(self, first, count, ref_slot=-1, ref_density=None, minr=0.0, maxr=2.0):
        r = None if ref_density is None else np.ascontiguousarray(ref_density, dtype=np.complex64)
        call("spe_reshift", self.h, int(first), int(count), int(ref_slot),
             None if r is None else r.view(np.float32).ctypes.data_as(_fp), float(minr), float(maxr))

    def average(self, first, count, errors, fraction, out_slot):
        err = np.ascontiguousarray(errors, dtype=np.float32)
        call("spe_average", self.h, int(first), int(count), fptr(err), float(fraction), int(out_slot))

    def average_module(self, first, count, errors, ft=True, fraction=1.0):
        err = np.ascontiguousarray(errors, dtype=np.float32)
        out = np.empty((self.n, self.n), np.float32)
        call("spe_average_module", self.h, int(first), int(count), fptr(err), int(bool(ft)), float(fraction), fptr(out))
        return out

    def crossover(self, first, count, errors, best_slot, avg_slot, dst_first, crossbalance, crossdiff,
                  crossexp=1.0, crossft=1.0, crosssym=False, use_average=0.0, update_support=True,
                  reality=0.0, minr=0.0, maxr=2.0):
        err = np.ascontiguousarray(errors, dtype=np.float32)
        call("spe_crossover", self.h, int(first), int(count), fptr(err), int(best_slot), int(avg_slot),
             int(dst_first), float(crossbalance), float(crossdiff), float(crossexp), float(crossft),
             int(bool(crosssym)), float(use_average), int(bool(update_support)), float(reality),
             float(minr), float(maxr))


def metrics_dict(m: SpeMetrics) -> dict:
    return {k: float(getattr(m, k)) for k, _ in SpeMetrics._fields_}


def crossover_draws(seed, order, suppdim, n, crossbalance, crossexp=1.0, crossft=1.0):
    """Host-only draws of the crossover (see include/spe_engine.h)."""
    order = np.ascontiguousarray(order, dtype=np.int32)
    count = len(order)
    draws = np.empty((count, 11), np.int32)
    rot = np.empty(count, np.float32)
    used = C.c_int32()
    args = [C.c_uint32(int(seed) & 0xFFFFFFFF), count, iptr(order), float(suppdim), int(n), float(crossbalance),
            float(crossexp), float(crossft), iptr(draws), fptr(rot)]
    call("spe_crossover_draws", *args, None, 0, C.byref(used))
    cm = np.empty(max(used.value, 1), np.int32)
    call("spe_crossover_draws", *args, iptr(cm), cm.size, C.byref(used))
    return draws, rot, cm[:used.value]


def prepare_pattern(intensities, center=(-1, -1), use_bounds=True):
    """Host pattern encoding of the reference Solver (see include/spe_engine.h)."""
    x = np.ascontiguousarray(intensities, dtype=np.float32)
    if x.ndim != 2 or x.shape[0] != x.shape[1]:
        raise ValueError("patterns must be square 2D arrays")
    out = np.empty_like(x)
    call("spe_prepare_pattern", fptr(x), x.shape[0], int(center[0]), int(center[1]),
         int(bool(use_bounds)), fptr(out))
    return out
