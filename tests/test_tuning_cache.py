"""The tuning cache file: the library's table of launch-shape choices is
exported and imported whole (checked before anything is recorded), the
window sigmas travel with it, a fresh process that loads the file uses the
saved choices, and choices recorded for a workload are reused without
timing. Host logic only: the forms and matrices here have no cells or
rows (the table is keyed by their sizes), so nothing reaches a GPU."""

import ctypes as C
import json
import os
import subprocess
import sys
import types

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture
def tune(capi):
    from dolfinx_gb300 import autotune

    autotune.clear()
    yield autotune
    autotune.clear()


def _form(capi, kind=0, degree=2, num_cells=0, k2=0.0):
    return capi.Form(kind, degree, num_cells, 0, None, None, None, None, 1.0, k2, 0.3, None,
                     (C.c_double * 3)())


def _csr(capi, nrows=0, nnz=0):
    return capi.Csr(nrows, nrows, 1, capi.F64, nnz, None, None, None)


def _matrix(nrows, nnz):
    """What the sigma table reads of a MatrixCSR: its shape and device."""
    return types.SimpleNamespace(nrows=nrows, nnz=nnz, vals=torch.zeros(0))


def _cpb(capi, form, mode):
    v = C.c_int32(0)
    capi.check(capi.lib().dfx_get_cells_per_block(C.byref(form), mode, C.byref(v)))
    return v.value


def _lanes(capi, A):
    v = C.c_int32(0)
    capi.check(capi.lib().dfx_get_spmv_lanes(C.byref(A), C.byref(v)))
    return v.value


def _record_some(capi, tune):
    L = capi.lib()
    f, fm, e = _form(capi), _form(capi, k2=1.0), _form(capi, kind=capi.FORM_ELASTICITY)
    capi.check(L.dfx_set_cells_per_block(C.byref(f), 0, 64))
    capi.check(L.dfx_set_cells_per_block(C.byref(fm), 1, 16))
    capi.check(L.dfx_set_cells_per_block(C.byref(e), 0, 8))
    A = _csr(capi)
    capi.check(L.dfx_set_spmv_lanes(C.byref(A), 16))
    tune.pin_sigma(_matrix(100, 2000), 256)
    return f, fm, e, A


def test_export_import_round_trip(capi, tune):
    L = capi.lib()
    f, fm, e, A = _record_some(capi, tune)
    n = C.c_int64(0)
    capi.check(L.dfx_tune_export(None, 0, C.byref(n)))
    assert n.value == 4
    small = np.zeros((2, 6), np.int64)
    assert L.dfx_tune_export(small.ctypes.data, 2, C.byref(n)) == capi.DFX_ERR_NO_MEMORY
    assert n.value == 4
    rows = tune._table()
    assert rows.shape == (4, 6)
    assert sorted(rows[:, 5].tolist()) == [8, 16, 16, 64]
    key = tune.assembly_key(fm, 1)
    assert [0, 1, 0, key, 0, 16] in rows.tolist()
    capi.check(L.dfx_tune_clear())
    assert _cpb(capi, f, 0) == 32 and _lanes(capi, A) != 16
    capi.check(L.dfx_tune_import(rows.ctypes.data, len(rows)))
    assert _cpb(capi, f, 0) == 64 and _cpb(capi, fm, 1) == 16 and _cpb(capi, e, 0) == 8
    assert _cpb(capi, fm, 0) == 32  # other mode: not recorded
    assert _lanes(capi, A) == 16
    assert np.array_equal(tune._table(), rows)


@pytest.mark.parametrize("bad", [
    [0, 3, 600, 36, 0, 32],     # unknown kind of choice
    [0, 1, 600, 36, 0, 48],     # not a cells-per-block candidate
    [0, 1, 600, 16 + 8, 0, 32],  # elasticity takes 2, 4 or 8
    [0, 2, 100, 2000, 4, 3],    # lanes per row
    [-1, 2, 100, 2000, 4, 8],   # device
])
def test_import_refuses_a_bad_row_and_records_nothing(capi, tune, bad):
    good = [0, 2, 100, 2000, 4, 8]
    rows = np.array([good, bad], np.int64)
    assert capi.lib().dfx_tune_import(rows.ctypes.data, 2) == capi.DFX_ERR_INVALID
    assert "tuning row 1" in capi.lib().dfx_last_error().decode()
    assert len(tune._table()) == 0


def test_save_and_load(capi, tune, tmp_path):
    f, fm, e, A = _record_some(capi, tune)
    path = str(tmp_path / "tuning.json")
    assert tune.save(path) == 5
    doc = json.loads(open(path).read())
    assert doc["format"] == "dfx-tuning" and doc["version"] == 1
    assert doc["sigma"] == [[0, 100, 2000, 256]]
    tune.clear()
    assert tune.recorded_sigma(_matrix(100, 2000)) is None
    assert tune.load(path) == 5
    assert _cpb(capi, f, 0) == 64 and _cpb(capi, e, 0) == 8 and _lanes(capi, A) == 16
    assert tune.recorded_sigma(_matrix(100, 2000)) == 256
    assert tune.recorded_sigma(_matrix(100, 2001)) is None
    assert tune.recorded_cells_per_block(fm, 1) == 16
    assert tune.recorded_cells_per_block(fm, 0) is None


def test_load_refuses_other_files(capi, tune, tmp_path):
    p = tmp_path / "x.json"
    p.write_text(json.dumps({"format": "something else"}))
    with pytest.raises(ValueError, match="not a tuning cache file"):
        tune.load(str(p))
    p.write_text(json.dumps({"format": "dfx-tuning", "version": 99}))
    with pytest.raises(ValueError, match="version 99"):
        tune.load(str(p))
    base = {"format": "dfx-tuning", "version": 1, "devices": {"0": None}}
    p.write_text(json.dumps(dict(base, choices=[[0, 1, 600, 36, 0]])))
    with pytest.raises(ValueError, match="6 integers"):
        tune.load(str(p))
    # a bad sigma and a bad choice each leave everything unrecorded
    p.write_text(json.dumps(dict(base, choices=[[0, 2, 100, 2000, 4, 8]],
                                 sigma=[[0, 100, 2000, 100]])))
    with pytest.raises(ValueError, match="bad sigma"):
        tune.load(str(p))
    p.write_text(json.dumps(dict(base, choices=[[0, 2, 100, 2000, 4, 7]],
                                 sigma=[[0, 100, 2000, 64]])))
    with pytest.raises(capi.DfxError):
        tune.load(str(p))
    assert len(tune._table()) == 0 and tune.recorded_sigma(_matrix(100, 2000)) is None


def test_load_skips_choices_of_another_device(capi, tune, tmp_path, monkeypatch):
    p = tmp_path / "t.json"
    doc = {"format": "dfx-tuning", "version": 1, "devices": {"0": "GPU A", "1": "GPU B"},
           "choices": [[0, 2, 100, 2000, 4, 8], [1, 2, 100, 2000, 4, 32]],
           "sigma": [[0, 100, 2000, 64], [1, 100, 2000, 1024]]}
    p.write_text(json.dumps(doc))
    monkeypatch.setattr(tune, "_device_names", lambda: {0: "GPU A", 1: "GPU C"})
    assert tune.load(str(p)) == 2  # device 1 is another model now
    assert tune._table()[:, 0].tolist() == [0]
    tune.clear()
    monkeypatch.setattr(tune, "_device_names", lambda: {0: "GPU A"})
    assert tune.load(str(p), check_devices=False) == 4
    tune.clear()
    monkeypatch.setattr(tune, "_device_names", lambda: {})
    assert tune.load(str(p)) == 4  # no GPU here: nothing to compare against


def test_recorded_choices_are_reused_without_timing(capi, tune):
    """tune_assembly / tune_sigma with reuse=True return a recorded choice
    before any device work (the objects here have no device data)."""
    f = _form(capi)
    asm = types.SimpleNamespace(form=f, mode=0)
    capi.check(capi.lib().dfx_set_cells_per_block(C.byref(f), 0, 16))
    res = tune.tune_assembly(asm, reuse=True)
    assert res == {"cells_per_block": 16, "ms": None, "recorded": True}
    M = _matrix(100, 2000)
    tune.pin_sigma(M, 1024)
    assert tune.tune_sigma(M, reuse=True) == {"sigma": 1024, "candidates": None,
                                              "recorded": True}
    tune.pin_sigma(M, 0)
    assert tune.recorded_sigma(M) is None
    with pytest.raises(ValueError):
        tune.pin_sigma(M, 100)


_LOAD_SCRIPT = r"""
import ctypes as C, sys
sys.path.insert(0, sys.argv[1])
from dolfinx_gb300 import _capi, autotune
f = _capi.Form(0, 2, 0, 0, None, None, None, None, 1.0, 0.0, 0.3, None, (C.c_double * 3)())
v = C.c_int32(0)
_capi.check(_capi.lib().dfx_get_cells_per_block(C.byref(f), 0, C.byref(v)))
before = v.value
n = autotune.load(sys.argv[2])
_capi.check(_capi.lib().dfx_get_cells_per_block(C.byref(f), 0, C.byref(v)))
print(before, n, v.value)
"""


def test_a_fresh_process_uses_the_saved_choices(capi, tune, tmp_path):
    _record_some(capi, tune)
    path = tmp_path / "tuning.json"
    tune.save(str(path))
    script = tmp_path / "load.py"
    script.write_text(_LOAD_SCRIPT)
    out = subprocess.run([sys.executable, str(script), ROOT, str(path)], check=True,
                         capture_output=True, text=True, timeout=120).stdout.split()
    assert out == ["32", "5", "64"]
