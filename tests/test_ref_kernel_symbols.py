"""The symbol table that loads the reference's compiled kernels
(baseline/ref_kernels.py) against the reference's source: every mangled name
demangles to a __global__ kernel of src/gpu/gpu_context.cu with that name and
that parameter list (CUDA_COMPLEX = float2, FLOAT = float, SUPPORTTYPE = int),
so the tests and the benchmark launch the kernels they mean.  Needs the
reference checkout and c++filt; no GPU."""
import re
import shutil
import subprocess

import pytest

from baseline import ref_kernels

SRC = ref_kernels.DEFAULT_REF / "src" / "gpu" / "gpu_context.cu"
pytestmark = pytest.mark.skipif(not SRC.exists() or shutil.which("c++filt") is None,
                                reason="needs the reference checkout and c++filt")

MACROS = {"CUDA_COMPLEX": "float2", "FLOAT": "float", "SUPPORTTYPE": "int", "cufftComplex": "float2"}


def _norm_type(decl):
    """Type of one parameter declaration, with the reference's macros
    expanded and the parameter name dropped."""
    decl = re.sub(r"/\*.*?\*/", " ", decl).strip()
    m = re.match(r"^(.*?)(\w+)\s*$", decl)
    t = m.group(1) if m and ("*" in m.group(1) or m.group(1).strip()) else decl
    t = t.replace("*", " * ")
    words = [MACROS.get(w, w) for w in t.split()]
    return "".join(w for w in words if w != "const")


def _kernels():
    text = SRC.read_text(errors="replace")
    out = {}
    for m in re.finditer(r"__global__\s+void\s+(\w+)\s*\(([^)]*)\)", text):
        params = [p for p in m.group(2).split(",") if p.strip()]
        out.setdefault(m.group(1), []).append([_norm_type(p) for p in params])
    return out


def _demangled(sym):
    r = subprocess.run(["c++filt", sym], capture_output=True, text=True, check=True)
    m = re.match(r"^(\w+)\((.*)\)$", r.stdout.strip())
    assert m, (sym, r.stdout)
    return m.group(1), [p.replace(" ", "") for p in m.group(2).split(",") if p.strip()]


@pytest.mark.parametrize("key", sorted(ref_kernels.SYMBOLS))
def test_symbol_names_a_kernel_of_the_reference(key):
    name, params = _demangled(ref_kernels.SYMBOLS[key])
    kernels = _kernels()
    assert name in kernels, name
    assert params in kernels[name], (name, params, kernels[name])
