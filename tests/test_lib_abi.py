"""The C-ABI library builds, loads and exports every entry point its header declares (no GPU needed)."""

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(etg_\w+)\s*\(", text, flags=re.M))
    return names


def test_header_declares_the_abi():
    names = declared_functions()
    assert {"etg_last_error", "etg_update_h_te", "etg_update_e_te", "etg_accumulate_dft",
            "etg_sim_create", "etg_sim_advance"} <= names  # fmt: skip


def test_library_exports_every_declared_symbol():
    from etalon_gb300 import _lib, build

    build.build()
    lib = _lib.lib()
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert missing == []
    assert set(_lib.SIGNATURES) | {"etg_last_error"} >= declared_functions()


def test_version_and_error_string_without_gpu():
    from etalon_gb300 import _lib

    lib = _lib.lib()
    assert lib.etg_version() >> 16 == 1
    assert isinstance(_lib.last_error(), str)


def test_bad_arguments_fail_before_touching_the_device():
    import ctypes as C

    from etalon_gb300 import _lib

    with pytest.raises(ValueError, match="dtype"):
        _lib.call("etg_sim_create", C.byref(C.c_void_p()), 3, 10, 10)
    with pytest.raises(ValueError, match="out of range"):
        _lib.call("etg_sim_create", C.byref(C.c_void_p()), 4, 1, 10)
    with pytest.raises(ValueError, match="out of range"):  # rows past the one-step kernels' launch grid
        _lib.call("etg_sim_create", C.byref(C.c_void_p()), 4, 262137, 10)
    with pytest.raises(ValueError):
        _lib.call("etg_update_h_te", 4, 0, 5, *([None] * 11), 1.0, 1.0, 1.0)
    with pytest.raises(ValueError, match="size"):  # rows past the launch grid
        _lib.call("etg_update_e_te", 4, 524273, 5, *([None] * 13), 1.0, 1.0)


def test_injected_fault_is_reported(monkeypatch):
    import ctypes as C

    from etalon_gb300 import _lib

    monkeypatch.setenv("ETG_FAULT", "etg_sim_create")
    with pytest.raises(_lib.EtgError, match="fault injected") as err:
        _lib.call("etg_sim_create", C.byref(C.c_void_p()), 4, 10, 10)
    assert err.value.code == _lib.ERR_INJECTED


def test_injected_fault_in_the_3d_create_is_reported(monkeypatch):
    import ctypes as C

    from etalon_gb300 import _lib

    monkeypatch.setenv("ETG_FAULT", "etg_yee3d_create")
    h = C.c_void_p()
    with pytest.raises(_lib.EtgError, match="fault injected") as err:
        _lib.call("etg_yee3d_create", C.byref(h), 4, 8, 8, 8, 0)
    assert err.value.code == _lib.ERR_INJECTED and h.value is None


@pytest.mark.parametrize(
    "name,args,words",
    [
        ("etg_sum_sq", (3, 4, 4, 4, 1, None, "OUT"), "dtype"),      # dtype must be 4 or 8
        ("etg_sum_sq", (4, 4, 4, 4, None, None, None), "bad arguments"),
        ("etg_block_mean", (4, 8, 8, 8, 1, 0, 2, 4, 1), "bad arguments"),  # block of 0 rows
        ("etg_block_mean", (4, 8, 8, 8, 1, 2, 2, 2, 1), "dtypes"),
        ("etg_cast", (4, 2, 8, 1, 1), "dtypes"),
        ("etg_sim_rasterize_cb", (None, 0.0, 0.0, 0.02, 0.02, 1e-16, 8.85e-12, 1.0, 0, None), "bad arguments"),
        ("etg_sim_get_cb", (None, 0, None), "bad arguments"),
        ("etg_sim_set_cb_window", (None, 0, 0, 1, 0, 1, None), "bad arguments"),
        ("etg_yee3d_create", ("HANDLE", 3, 8, 8, 8, 0), "bad arguments"),      # dtype must be 4 or 8
        ("etg_yee3d_create", ("HANDLE", 4, 8, 8, 0, 0), "bad arguments"),      # empty axis
        ("etg_yee3d_create", ("HANDLE", 4, 8, 8, 8, 8), "bad arguments"),      # periodic mask of 3 bits
        ("etg_yee3d_create", (None, 4, 8, 8, 8, 0), "bad arguments"),
        ("etg_yee3d_create", ("HANDLE", 8, 70000, 8, 8, 0), "too large"),
        ("etg_yee3d_create", ("HANDLE", 4, 60000, 60000, 60000, 0), "too large"),
        ("etg_yee3d_create", ("HANDLE", 4, 1, 400000, 10000, 0), "too large"),  # row offsets past 32 bits
        ("etg_yee3d_create", ("HANDLE", 4, 1, 500000, 8, 0), "too large"),      # rows past the launch grid
        ("etg_yee3d_set_scalars", (None, None), "null argument"),
        ("etg_yee3d_set_profile", (None, 0, None, None, None, None, None, None), "bad arguments"),
        ("etg_yee3d_set_field", (None, 0, None), "bad field id"),
        ("etg_yee3d_get_field", (None, 0, None), "bad field id"),
        ("etg_yee3d_add_source", (None, 0, 1, None, 0, 1, None), "bad arguments"),
        ("etg_yee3d_add_monitor", (None, 0, 1, None, 1, 0, 1, None), "bad arguments"),
        ("etg_yee3d_get_dft", (None, 0, None), "bad monitor"),
        ("etg_yee3d_advance", (None, 1), "bad arguments"),
        ("etg_yee3d_synchronize", (None,), "null handle"),
        ("etg_yee3d_step_index", (None, None), "null argument"),
        ("etg_yee3d_last_timing", (None, None, None), "null argument"),
        ("etg_yee3d_kernel_timing", (None, 1, None, None), "bad arguments"),
        ("etg_yee3d_set_option", (None, 0, 1), "bad option"),
    ],
)  # fmt: skip
def test_entry_points_reject_bad_arguments_before_touching_the_gpu(name, args, words):
    """Argument checks come first, so they hold (ValueError with the reason) on any machine."""
    import ctypes as C

    from etalon_gb300 import _lib

    out, handle = C.c_double(), C.c_void_p()
    args = tuple(C.byref(out) if a == "OUT" else C.byref(handle) if a == "HANDLE" else a for a in args)
    with pytest.raises(ValueError, match=words):
        _lib.call(name, *args)
