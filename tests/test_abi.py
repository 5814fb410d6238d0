"""C ABI checks that need no GPU: the library loads, exports every declared
symbol, and rejects bad configurations without touching a device."""
import ctypes as ct
import subprocess

import pytest

from iqtree2_gb300 import engine


def test_library_exports_every_declared_symbol():
    L = engine.lib()
    names = engine.exported_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", engine.library_path()], capture_output=True, text=True).stdout
    for n in names:
        assert f" T {n}" in out, n


def test_memory_required_and_bad_config():
    need = engine.Engine.memory_required(nptn=50000, nstates=20, ncat=4, ntaxa=100, state_unknown=23, nslots=294)
    # 294 slots * 80 doubles * 50048 padded patterns dominate
    assert need >= 294 * 80 * 50048 * 8
    with pytest.raises(engine.EngineError) as ei:
        engine.Engine.memory_required(nptn=10, nstates=65, ncat=4, ntaxa=5, state_unknown=65, nslots=9)
    assert ei.value.code == 1


def test_create_without_gpu_reports_no_device():
    cfg = engine.Config(100, 4, 4, 5, 18, 9, 0, 0, 0, 10)
    h = ct.c_void_p()
    rc = engine.lib().iqgpu_create(ct.byref(cfg), ct.byref(h))
    if rc == 0:  # running on a GB300 host: nothing to check here
        engine.lib().iqgpu_destroy(h)
        pytest.skip("a GPU is present")
    assert rc == 7  # IQGPU_ERR_NODEV
    assert b"device" in engine.lib().iqgpu_last_error()


def test_reference_safe_rule_in_memory_sizing():
    """The engine applies the reference's SAFE rule (tree/phylotreesse.cpp:95-96)
    at configuration: a 61-state FP64 engine keeps one scale count per pattern
    x category even when NORM is asked for, unless IQGPU_FLAG_SAFE_AS_GIVEN."""
    kw = dict(nptn=10000, nstates=61, ncat=4, ntaxa=40, state_unknown=61, nslots=114)
    norm, safe = engine.Engine.memory_required(safe=0, **kw), engine.Engine.memory_required(safe=1, **kw)
    assert norm == safe
    given = engine.Engine.memory_required(safe=0, flags=engine.FLAG_SAFE_AS_GIVEN, **kw)
    assert safe - given >= 114 * 3 * 10000  # the per-category counts
    kw20 = dict(kw, nstates=20, state_unknown=23)
    assert engine.Engine.memory_required(safe=0, **kw20) < engine.Engine.memory_required(safe=1, **kw20)
    kw_big = dict(kw20, ntaxa=2000, nslots=5994, nptn=64)
    assert engine.Engine.memory_required(safe=0, **kw_big) == engine.Engine.memory_required(safe=1, **kw_big)
