"""The C-ABI library builds, loads and exports its header; host-side logic (CPU)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from chemsim_gb300 import _lib
from chemsim_gb300.workloads import (batch_specs, channel_spec, circles_mask,
                                     splitmix64, taylor_green, uniform)


def test_library_exports_every_header_symbol(cuda_lib):
    declared = _lib.header_functions()
    assert "lbm_create" in declared and "lbm_step" in declared
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared:
        assert getattr(cuda_lib, n) is not None


def test_every_header_function_has_a_signature():
    declared = set(_lib.header_functions())
    assert declared <= set(_lib.SIGNATURES), declared - set(_lib.SIGNATURES)


def _header_arities():
    """Parameter count of every function declared in include/*.h."""
    import os
    import re
    out = {}
    for fn in sorted(os.listdir(_lib.HEADER_DIR)):
        if not fn.endswith(".h"):
            continue
        text = re.sub(r"/\*.*?\*/", "", open(os.path.join(_lib.HEADER_DIR, fn)).read(), flags=re.S)
        for m in re.finditer(r"\b(lbm_\w+)\s*\(([^)]*)\)\s*;", text):
            args = m.group(2).strip()
            out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


CRATE = os.path.join(os.path.dirname(_lib.HEADER_DIR), "lbm-cuda")


def test_rust_binding_declares_every_entry_point():
    """The extern block of the lbm-cuda crate (lbm-cuda/src/lib.rs) names
    every function of the header with the same number of parameters, and
    nothing else."""
    import re
    text = open(os.path.join(CRATE, "src", "lib.rs")).read()
    block = text[text.index('extern "C" {'):]
    block = block[:block.index("\n    }\n")]
    rust = {m.group(1): (0 if not m.group(2).strip() else m.group(2).count(",") + 1)
            for m in re.finditer(r"pub fn (lbm_\w+)\(([^)]*)\)", block, re.S)}
    header = _header_arities()
    assert set(header) == set(_lib.header_functions())
    assert set(rust) == set(header), (set(header) ^ set(rust))
    wrong = {n: (header[n], rust[n]) for n in header if header[n] != rust[n]}
    assert not wrong, wrong


def test_rust_structs_and_constants_match_the_header():
    """lbm_health / lbm_desc field order and the LBM_* constants of the
    crate are those of include/lbm_cuda.h."""
    import re
    header = re.sub(r"/\*.*?\*/", "", open(os.path.join(_lib.HEADER_DIR, "lbm_cuda.h")).read(),
                    flags=re.S)
    rust = open(os.path.join(CRATE, "src", "lib.rs")).read()
    for cname, rname in (("lbm_health", "LbmHealth"), ("lbm_desc", "LbmDesc")):
        body = re.search(r"typedef struct %s \{(.*?)\}" % cname, header, re.S).group(1)
        cfields = re.findall(r"(\w+)\s*(?:,|;)", body.replace("*", " "))
        rbody = re.search(r"pub struct %s \{(.*?)\}" % rname, rust, re.S).group(1)
        rfields = re.findall(r"pub (\w+):", rbody)
        assert cfields == rfields, (cname, cfields, rfields)
    consts = dict(re.findall(r"#define (LBM_\w+)\s+\(?(-?(?:0x)?[0-9a-fA-F]+)\)?", header))
    rconsts = dict(re.findall(r"pub const (LBM_\w+): c_int = (-?(?:0x)?[0-9a-fA-F]+);", rust))
    assert rconsts, "no constants in the crate"
    for name, val in rconsts.items():
        assert int(consts[name], 0) == int(val, 0), name
    missing = {n for n in consts if n.startswith(("LBM_ERR", "LBM_F", "LBM_X", "LBM_Y", "LBM_COLL",
                                                 "LBM_RENDER", "LBM_SOLID"))} - set(rconsts)
    assert not missing, missing


def test_rust_build_script_and_chemsim_patch():
    """build.rs compiles the library's own CUDA sources for sm_103a (or links
    the prebuilt .so); chemsim.patch is a unified diff against chemsim that
    routes State's step, moments and health through the crate."""
    build = open(os.path.join(CRATE, "build.rs")).read()
    assert "arch=compute_103a,code=sm_103a" in build and ".cuda(true)" in build
    assert "LBM_CUDA_DIR" in build and '"cu"' in build
    cargo = open(os.path.join(CRATE, "Cargo.toml")).read()
    assert 'name = "lbm-cuda"' in cargo and "cc =" in cargo
    patch = open(os.path.join(CRATE, "chemsim.patch")).read()
    files = [l.split()[1] for l in patch.splitlines() if l.startswith("+++ ")]
    assert files == ["b/Cargo.toml", "b/src/lbm.rs", "b/src/lib.rs", "b/src/main.rs"]
    added = "\n".join(l[1:] for l in patch.splitlines() if l.startswith("+") and not l.startswith("+++"))
    for needle in ("dev.step(1)", "dev.moments()", "dev.health()", "fn initial_device",
                   "fn set_geometry", "extern crate lbm_cuda", "State::initial_device"):
        assert needle in added, needle
    # every hunk header's line counts agree with its body
    import re
    for m in re.finditer(r"^@@ -\d+,(\d+) \+\d+,(\d+) @@.*?\n(.*?)(?=^@@|^diff |\Z)", patch,
                         re.S | re.M):
        body = m.group(3).splitlines()
        old = sum(1 for l in body if l[:1] in (" ", "-"))
        new = sum(1 for l in body if l[:1] in (" ", "+"))
        assert (old, new) == (int(m.group(1)), int(m.group(2))), m.group(0)[:80]


def test_version_and_error_string(cuda_lib):
    assert cuda_lib.lbm_version() >= 100
    assert isinstance(_lib.last_error(), str)


@pytest.mark.parametrize("args,needle", [
    ((0, 8, 1.0, 0, 0), "sides"),
    ((8, 300000, 1.0, 0, 0), "sides"),
    ((8, 8, 0.0, 0, 0), "tau"),
    ((8, 8, float("nan"), 0, 0), "tau"),
    ((8, 8, 1.0, 9, 0), "precision"),
    ((8, 8, 1.0, 0, 0x3), "flags"),
    ((8, 8, 1.0, 0, 0x100), "flags"),
])
def test_create_rejects_bad_arguments(cuda_lib, args, needle):
    """Argument checks happen before any device call (no GPU needed)."""
    h = ctypes.c_void_p()
    rc = cuda_lib.lbm_create(*args, ctypes.byref(h))
    assert rc == _lib.LBM_ERR_INVALID_ARGUMENT
    assert needle in _lib.last_error()
    assert not h.value


def test_null_handles_are_rejected(cuda_lib):
    assert cuda_lib.lbm_destroy(None) == _lib.LBM_OK
    for fn, extra in [("lbm_step", (1,)), ("lbm_set_force", (0.0, 0.0)),
                      ("lbm_set_populations", (None,)), ("lbm_check", (None,)),
                      ("lbm_synchronize", ()), ("lbm_set_tile", (0, 0))]:
        rc = getattr(cuda_lib, fn)(None, *extra)
        assert rc == _lib.LBM_ERR_INVALID_ARGUMENT, fn
    assert cuda_lib.lbm_create(8, 8, 1.0, 0, 0, None) == _lib.LBM_ERR_INVALID_ARGUMENT


def test_check_raises_lbm_error(cuda_lib):
    with pytest.raises(_lib.LBMError) as ei:
        _lib.check(cuda_lib.lbm_step(None, 1))
    assert ei.value.status == _lib.LBM_ERR_INVALID_ARGUMENT


def test_splitmix64_known_answer():
    # The first output of splitmix64 seeded with 0 (Vigna's reference).
    assert int(splitmix64(0, 0, 1)[0]) == 0xE220A8397B1DCDAF
    a = uniform(7, 100, 1000)
    assert a.min() >= 0 and a.max() < 1
    np.testing.assert_array_equal(a, uniform(7, 100, 1000))


def test_workloads_shapes_and_determinism():
    rho, ux, uy = taylor_green(32, 16)
    assert rho.shape == (16, 32) and rho.dtype == np.float32
    assert abs(float(rho.mean()) - 1.0) < 1e-4
    # divergence-free in the XY frame (central differences, periodic)
    dx = 2 * np.pi / 32 * 2     # central-difference spans two cells
    dy = 2 * np.pi / 16 * 2
    div = (np.roll(ux, -1, 1) - np.roll(ux, 1, 1)) / np.sin(dx / 2) * (dx / 2) / 2 \
        + (np.roll(uy, -1, 0) - np.roll(uy, 1, 0)) / np.sin(dy / 2) * (dy / 2) / 2
    assert np.max(np.abs(div)) < 1e-7
    m1 = circles_mask(200, 100, 5, 4, 9, seed=3)
    m2 = circles_mask(200, 100, 5, 4, 9, seed=3)
    np.testing.assert_array_equal(m1, m2)
    assert 0 < m1.mean() < 0.5
    spec = channel_spec(256, n_obstacles=4, r_lo=4, r_hi=8)
    assert spec.solid.shape == (256, 256) and spec.force == (1e-6, 0.0)
    specs = batch_specs(8, lo=16, hi=64)
    assert len(specs) == 8
    for s in specs:
        assert 16 <= s.w <= 64 and 16 <= s.h <= 64 and 0.52 <= s.tau <= 1.0


def test_mirror_asserts_like_the_reference():
    from chemsim_gb300.lbm import D2Q9, Discretization, TRT
    with pytest.raises(AssertionError):
        D2Q9([np.zeros((2, 2))] * 8)
    with pytest.raises(AssertionError):
        D2Q9([np.zeros((2, 2))] * 8 + [np.zeros((3, 2))])
    disc = Discretization(1.0, 1.0)
    assert abs(disc.isothermal_speed_of_sound() - 1 / np.sqrt(3)) < 1e-7
    t = TRT.new(0.25, 0.1, disc)
    assert abs(t.kinematic_shear_viscosity(disc) - 0.1) < 1e-6
