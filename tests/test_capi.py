"""The C ABI library loads without a GPU and exports every declared symbol."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(nexus_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "nexus_ntt_forward" in names and "nexus_context_create" in names


def test_library_exports_every_declared_symbol():
    from nexus_gb300 import _lib
    lib = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound, set(declared_functions()) - bound


def test_context_rejects_bad_arguments_without_gpu():
    # argument validation happens before any CUDA call
    from nexus_gb300 import _lib
    lib = _lib.lib()
    h = ctypes.c_void_p()
    arr = (ctypes.c_uint64 * 2)(3, 5)
    assert lib.nexus_context_create(5, arr, 2, ctypes.byref(h)) != 0
    assert b"log_n" in lib.nexus_last_error()
    assert lib.nexus_ntt_forward(None, None, 1, 0, 1, None) != 0
    assert b"null" in lib.nexus_last_error()


def test_lockstep_and_hoisting_entry_points_reject_null_arguments_without_gpu():
    # every check below runs before any device work
    from nexus_gb300 import _lib
    lib = _lib.lib()
    one = (ctypes.c_void_p * 1)(None)
    steps = (ctypes.c_int * 1)(1)
    cases = [
        ("nexus_switch_key_batch", lambda: lib.nexus_switch_key_batch(None, None, 1, 1, None, None, None), b"null"),
        ("nexus_rotate_vector_many", lambda: lib.nexus_rotate_vector_many(None, None, steps, 1, one), b"null"),
        ("nexus_rotate_vector_many_batch",
         lambda: lib.nexus_rotate_vector_many_batch(None, one, 1, steps, 1, one), b"null"),
        ("nexus_evaluator_set_hoisting", lambda: lib.nexus_evaluator_set_hoisting(None, 1), b"null"),
        ("nexus_argmax_batch", lambda: lib.nexus_argmax_batch(None, one, 1, 4, one), b"null"),
        ("nexus_bootstrapper_stage_batch", lambda: lib.nexus_bootstrapper_stage_batch(None, 0, one, None, 1, one, one),
         b"null"),
        ("nexus_autotune", lambda: lib.nexus_autotune(None, 1, 1, 1, None, None, None), b"null"),
        ("nexus_set_tuning", lambda: lib.nexus_set_tuning(None, 0, 0), b"null"),
        ("nexus_set_ntt_form", lambda: lib.nexus_set_ntt_form(None, 1), b"null"),
        ("nexus_get_ntt_form", lambda: lib.nexus_get_ntt_form(None, None), b"null"),
    ]
    for name, call, word in cases:
        assert call() != 0, name
        msg = lib.nexus_last_error()
        assert msg.startswith(name.encode()) and word in msg, (name, msg)


def test_keyswitch_workload_rejects_a_level_outside_the_chain_without_gpu():
    import subprocess
    import sys
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--workload", "keyswitch", "--ks-limbs", "40"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "--ks-limbs" in r.stderr


def test_graph_and_tensor_rate_entry_points_reject_bad_arguments_without_gpu():
    # every check below runs before any CUDA call
    from nexus_gb300 import _lib
    lib = _lib.lib()
    out = ctypes.c_void_p()
    d = ctypes.c_double()
    cases = [
        ("nexus_graph_capture_begin", lambda: lib.nexus_graph_capture_begin(None), b"legacy default stream"),
        ("nexus_graph_capture_end", lambda: lib.nexus_graph_capture_end(None, ctypes.byref(out)), b"null"),
        ("nexus_graph_launch", lambda: lib.nexus_graph_launch(None, None), b"null graph"),
        ("nexus_graph_info", lambda: lib.nexus_graph_info(None, None, None, None), b"null graph"),
        ("nexus_tensor_rate", lambda: lib.nexus_tensor_rate(2, 10, ctypes.byref(d), None), b"kind"),
        ("nexus_tensor_rate", lambda: lib.nexus_tensor_rate(0, 0, ctypes.byref(d), None), b"rounds"),
        ("nexus_tensor_rate", lambda: lib.nexus_tensor_rate(0, 10, None, None), b"null"),
        ("nexus_tensor_tile", lambda: lib.nexus_tensor_tile(0, 1, None, None, None), b"null"),
    ]
    for name, call, word in cases:
        assert call() != 0, name
        msg = lib.nexus_last_error()
        assert msg.startswith(name.encode()) and word in msg, (name, msg)
    assert lib.nexus_graph_destroy(None) == 0


def test_graph_wrapper_needs_a_stream_without_gpu():
    from nexus_gb300.operators import Graph
    with pytest.raises(ValueError):
        Graph(None)


def test_memory_info_reports_an_error_without_a_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    import nexus_gb300 as ng
    with pytest.raises(ng.NexusError, match="nexus_memory_info"):
        ng.memory_info()
