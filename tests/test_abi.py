"""The C-ABI library: builds, loads, exports every declared symbol, and its
struct layouts match the ctypes mirror (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "madsdp_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(msdp_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    from madsdp_gpu import _lib
    assert sorted(n for n, _, _ in _lib.SIGNATURES) == names


def test_struct_layouts_match_header(built_lib):
    from madsdp_gpu import _lib
    probe = r'''
#include <stdio.h>
#include <stddef.h>
#include "madsdp_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(msdp_components), sizeof(msdp_options),
         sizeof(msdp_problem_desc), sizeof(msdp_stats), sizeof(msdp_iter_record));
  printf("%zu %zu %zu %zu\n", offsetof(msdp_components, tau), offsetof(msdp_options, switch_tol),
         offsetof(msdp_problem_desc, C_lin), offsetof(msdp_stats, n_predictor));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        cfile = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(cfile, "w").write(probe)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), cfile, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sizes = list(map(int, out[:5]))
    offs = list(map(int, out[5:]))
    assert sizes == [C.sizeof(_lib.Components), C.sizeof(_lib.Options), C.sizeof(_lib.ProblemDesc),
                     C.sizeof(_lib.Stats), C.sizeof(_lib.IterRecord)]
    assert offs == [_lib.Components.tau.offset, _lib.Options.switch_tol.offset,
                    _lib.ProblemDesc.C_lin.offset, _lib.Stats.n_predictor.offset]


def test_defaults_mirror_reference_components(built_lib):
    from madsdp_gpu import _lib
    lib = _lib.load()
    c = _lib.Components()
    lib.msdp_default_components(C.byref(c))
    # src/components.jl defaults
    assert (c.tau, c.shrink, c.boundary, c.sigma_exponent) == (0.95, 0.8, 0.95, 3.0)
    assert (c.initial_ratio, c.ratio, c.initial_shift, c.max_shift) == (0.25, 0.5, 1.0, 1e10)
    assert (c.dc_beta, c.dc_delta, c.dc_A, c.centering_max_iter) == (0.2, 1.0, 2.0, 50)
    o = _lib.Options()
    lib.msdp_default_options(C.byref(o))
    # src/options.jl:3-15
    assert (o.tol, o.max_iter, o.max_wall_time, o.mu_min) == (1e-7, 100, 3600.0, 1e-14)
    assert (o.regularize_schur, o.max_schur_reg, o.datasparsity) == (1e-12, 8, 8)


def test_context_without_device_fails_cleanly(built_lib):
    from madsdp_gpu import _lib
    lib = _lib.load()
    if lib.msdp_device_count() > 0:
        pytest.skip("a device is present")
    h = C.c_void_p()
    assert lib.msdp_context_create(0, C.byref(h)) != 0


def test_invalid_configurations_are_rejected_before_any_device_work():
    import madsdp_gpu as M
    with pytest.raises(ValueError):
        M.ScaledIdentity(0)
    with pytest.raises(ValueError):
        M.ScaledIdentity(float("nan"))
