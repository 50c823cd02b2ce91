"""``spring_core.GPUtils``: the device queries the reference's front end uses
to choose its GPUs (``spring/mpr.py:142-165``, ``MPR.SelectGPUs``).

Same functions and return types as the reference's binding
(``src/wrapper.cpp:459-484`` over ``src/gpu/gpu_utils.cu:13-94``):

* ``get_count()`` -> int: CUDA devices (0 without any);
* ``get_ids()`` -> list[int]: 0 .. count-1;
* ``get_info()`` -> list[str]: device names;
* ``get_usage()`` -> list[int]: GPU utilisation in percent per device, from
  the NVIDIA management library when it can be loaded, else -1 for every
  device (the reference built without NVML).

Where the reference asks NVML for "device i" by NVML's own enumeration
(which need not follow the CUDA ordinals, e.g. under CUDA_VISIBLE_DEVICES),
this module looks each CUDA device up by its PCI bus id, so ``get_usage()[i]``
always belongs to CUDA device i.  The queries only read: nothing here
changes a device setting.
"""
from __future__ import annotations

import ctypes as C

from .. import _lib


def get_count() -> int:
    return _lib.device_count()


def get_ids() -> list[int]:
    return list(range(get_count()))


def get_info() -> list[str]:
    return [_lib.device_info(i)[0] for i in range(get_count())]


class _Utilization(C.Structure):
    _fields_ = [("gpu", C.c_uint), ("memory", C.c_uint)]


def _nvml():
    for name in ("libnvidia-ml.so.1", "libnvidia-ml.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


def get_usage() -> list[int]:
    n = get_count()
    usage = [-1] * n
    if n == 0:
        return usage
    nvml = _nvml()
    if nvml is None:
        return usage
    init = getattr(nvml, "nvmlInit_v2", None) or getattr(nvml, "nvmlInit", None)
    by_bus = getattr(nvml, "nvmlDeviceGetHandleByPciBusId_v2", None) or \
        getattr(nvml, "nvmlDeviceGetHandleByPciBusId", None)
    util = getattr(nvml, "nvmlDeviceGetUtilizationRates", None)
    if init is None or by_bus is None or util is None or init() != 0:
        return usage
    try:
        for i in range(n):
            bus = _lib.device_info(i)[1].encode()
            handle = C.c_void_p()
            if by_bus(C.c_char_p(bus), C.byref(handle)) != 0:
                continue
            u = _Utilization()
            if util(handle, C.byref(u)) == 0:
                usage[i] = int(u.gpu)
    finally:
        nvml.nvmlShutdown()
    return usage
