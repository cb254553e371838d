"""CPU checks of the C-ABI boundary: the library builds, loads, and exports every
function include/apbf_gb300.h declares; the ctypes binding covers exactly that
set.  No compute call is made (this machine may have no GPU)."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "apbf_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(apbf_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_stage_api():
    names = declared_functions()
    for required in ("apbf_neighborhood_green_apply", "apbf_incompressibility_apply", "apbf_update_transfers_apply",
                     "apbf_particle_transfer_apply", "apbf_spread_kernel_width_apply", "apbf_substep",
                     "apbf_sort_pairs", "apbf_prefix_sum"):
        assert required in names


def test_library_exports_every_declared_symbol(native_lib):
    from apbf_gb300 import _native

    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (apbf_[a-z0-9_]+)$", out, flags=re.M))
    names = set(declared_functions())
    assert names <= exported, names - exported
    assert set(_native.SIGNATURES) == names
    for n in names:
        assert hasattr(native_lib, n)


def test_abi_version_and_defaults(native_lib):
    import ctypes as C

    from apbf_gb300 import _native

    assert native_lib.apbf_abi_version() == 1
    s = _native.Settings()
    native_lib.apbf_default_settings(C.byref(s))
    # source/settings.cpp:5-31
    assert s.height_kernel_id == 1 and s.gradient_kernel_id == 1
    assert s.solver_iterations == 3 and s.boundariness_calculation_method == 2
    assert abs(s.target_radius_scale_factor - 0.3) < 1e-7 and s.merge_duration == 2.0


def test_oracle_default_settings_match_library(native_lib):
    """The oracle's restated defaults (used by the bench's CPU legs, which must not load
    the product library) equal apbf_default_settings field for field."""
    import ctypes as C

    from apbf_gb300 import _native
    from oracle import oracle as o

    s = _native.Settings()
    native_lib.apbf_default_settings(C.byref(s))
    for f, _ in _native.Settings._fields_:
        if not f.startswith("pad"):
            assert abs(float(getattr(s, f)) - float(o.DEFAULT_SETTINGS[f])) < 1e-7, f


def test_struct_sizes_match_oracle():
    import ctypes as C

    from apbf_gb300 import _native
    from oracle import oracle as o

    assert C.sizeof(_native.Settings) == C.sizeof(o.OrSettings) == 96
    assert [f for f, _ in _native.Settings._fields_] == [f for f, _ in o.OrSettings._fields_]


def test_invalid_create_rejected_without_gpu(native_lib):
    import ctypes as C

    from apbf_gb300 import _native

    cfg = _native.Config(0, 0, 0, 0, 0)
    h = C.c_void_p()
    assert native_lib.apbf_create(C.byref(cfg), C.byref(h)) == 1  # APBF_ERR_INVALID_ARG before any CUDA call
    assert b"invalid capacities" in native_lib.apbf_last_error()
