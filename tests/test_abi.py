"""The C ABI: the library loads without a GPU and exports every entry point the
header declares, with C linkage. No compute is called here."""

from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

from diorama_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "diorama_gb300.h"


def declared_functions() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(dg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_reference_surface():
    names = declared_functions()
    for prefix in ("dg_prefix_sum_", "dg_radix_sort_", "dg_tile_rasterizer_", "dg_renderer_", "dg_training_loss_",
                   "dg_trainer_", "dg_buffer_", "dg_context_"):
        assert any(n.startswith(prefix) for n in names), prefix


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # Every binding this package uses is declared in the header too, and every
    # entry point the header declares has a ctypes signature here.
    undeclared = [n for n in _lib.SIGNATURES if n not in declared_functions()]
    assert not undeclared, undeclared
    unbound = [n for n in declared_functions() if n != "dg_status" and n not in _lib.SIGNATURES]
    assert not unbound, unbound


def test_exports_have_c_linkage():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIBRARY)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for name in declared_functions():
        assert name in exported, f"{name} is not an unmangled export"


def test_error_string_and_version_without_gpu():
    lib = _lib.load()
    assert lib.dg_abi_version() == 1
    assert isinstance(lib.dg_last_error(), bytes)


def test_null_arguments_fail_with_a_status():
    lib = _lib.load()
    status = lib.dg_prefix_sum_encode(None)
    assert status == _lib.DG_ERROR_INVALID_ARGUMENT
    assert b"NULL" in lib.dg_last_error()
    out = ctypes.c_void_p()
    assert lib.dg_renderer_create(None, 0, ctypes.byref(out)) == _lib.DG_ERROR_INVALID_ARGUMENT


def test_node_addon_calls_only_declared_entry_points():
    """The Node-API addon (diorama_gb300/node/diorama.cc; not compiled here: node
    is absent) wraps only functions the header declares, and the TypeScript shims
    call only functions the addon registers."""
    root = HEADER.parent.parent / "diorama_gb300" / "node"
    addon = (root / "diorama.cc").read_text()
    called = set(re.findall(r"\b(dg_[a-z0-9_]+)\s*\(", addon))
    assert called and called <= set(declared_functions()), called - set(declared_functions())
    registered = set(re.findall(r'\{"([a-zA-Z]+)", nullptr,', addon))
    used = set()
    for ts in (root / "ts").glob("*.ts"):
        used |= set(re.findall(r"native\.([a-zA-Z]+)\(", ts.read_text()))
    assert used and used <= registered, used - registered
