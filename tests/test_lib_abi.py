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
    with pytest.raises(ValueError):
        _lib.call("etg_update_h_te", 4, 0, 5, *([None] * 11), 1.0, 1.0, 1.0)


def test_injected_fault_is_reported(monkeypatch):
    import ctypes as C

    from etalon_gb300 import _lib

    monkeypatch.setenv("ETG_FAULT", "etg_sim_create")
    with pytest.raises(_lib.EtgError, match="fault injected") as err:
        _lib.call("etg_sim_create", C.byref(C.c_void_p()), 4, 10, 10)
    assert err.value.code == _lib.ERR_INJECTED
