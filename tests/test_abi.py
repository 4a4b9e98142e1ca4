"""The C ABI library loads on a machine without a GPU and exports every
symbol include/bt.h declares; host-only entry points work without a GPU."""
import math
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "bt.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bt_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol(btlib):
    import initializator_gb300 as bt
    names = declared_symbols()
    assert names, "no declarations found"
    for n in names:
        assert hasattr(btlib, n), n
    assert sorted(bt.EXPORTS) == names
    out = subprocess.run(["nm", "-D", "--defined-only", bt.LIB_PATH], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\b", out), n


def test_version(btlib):
    assert b"sm_103a" in btlib.bt_version()


def test_create_rejects_bad_config(btlib):
    import ctypes
    import initializator_gb300 as bt
    cfg = bt.make_config((4, 4, 4), dx=1e-6, dt=1e-5)
    cfg.nx = 0
    h = ctypes.c_void_p()
    assert btlib.bt_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
    cfg = bt.make_config((4, 4, 4), dx=1e-6, dt=-1.0)
    assert btlib.bt_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
    cfg = bt.make_config((4, 4, 4), dx=1e-6, dt=1e-5, buffer=(3, 0, 0))
    assert btlib.bt_create(ctypes.byref(cfg), ctypes.byref(h)) == -1


def _sched(seq, n, **kw):
    import initializator_gb300 as bt
    return bt.sequence_schedule(seq, n, **kw)


def test_schedule_fid_and_inversion(btlib):
    d = (0.0, 0.0, 1.0)
    s = _sched(0, 10, dt=1e-5, direction=d)
    assert s == [(0, 2, 0.5 * math.pi, (1.0, 0.0, 0.0))]
    s = _sched(5, 10, dt=1e-5, direction=d)
    assert s == [(0, 2, math.pi, (1.0, 0.0, 0.0))]
    assert _sched(5, 10, dt=1e-5, direction=d, gpu_variant=False) == []


def test_schedule_cpmg_counts(btlib):
    dt = 1.0
    gpu = _sched(1, 200, dt=dt, time1=2.5, direction=(1, 0, 0))
    cpu = _sched(1, 300, dt=dt, time1=1.2, direction=(1, 0, 0), gpu_variant=False)
    assert len(gpu) == 1 + 20 and gpu[1][0] == 3 and gpu[2][0] == 8
    assert len(cpu) == 1 + 100
    assert all(p[1] == 2 and p[2] == math.pi for p in gpu[1:])


def test_schedule_pgse_9(btlib):
    dt = 1.0
    s = _sched(9, 60, dt=dt, time1=5.5, time2=20.0, direction=(0, 0, 1), gradient_pulse=0.3)
    assert [(p[0], p[1]) for p in s] == [(0, 2), (6, 1), (16, 2), (26, 1)]
    assert s[1][2] == 0.3 and s[1][3] == (0.0, 0.0, 1.0)
    assert s[2][2] == math.pi and s[2][3] == (1.0, 0.0, 0.0)


def test_schedule_98_99(btlib):
    mg = (1e-3, -2e-3, 3e-3)
    s98 = _sched(98, 60, dt=1.0, time1=5.5, time2=20.0, multiple_gradients=mg)
    assert [(p[0], p[1]) for p in s98] == [(0, 2), (6, 3), (16, 2), (26, 3)]
    assert s98[0][3] == (0.0, -1.0, 0.0) and s98[2][3] == (0.0, 0.0, 1.0)
    assert s98[1][3] == mg and s98[3][3] == mg
    s99 = _sched(99, 60, dt=1.0, time1=5.5, time2=20.0, multiple_gradients=mg)
    assert [(p[0], p[1]) for p in s99] == [(6, 3), (26, 3)]
    assert s99[1][3] == tuple(-v for v in mg)


def test_schedule_pfg_gpu_vs_cpu(btlib):
    kw = dict(dt=1.0, time1=3.3, time2=7.7, direction=(0, 0, 1), gradient_pulse=0.1)
    g = _sched(2, 40, **kw)
    c = _sched(2, 40, gpu_variant=False, **kw)
    assert [(p[0], p[1]) for p in g] == [(0, 2), (4, 1), (7, 2), (15, 2), (18, 1)]
    assert [p[0] for p in c] == [p[0] for p in g]
    assert g[0][3] == (-1.0, 0.0, 0.0) and c[0][3] == (1.0, 0.0, 0.0)
    assert g[3][3] == (-1.0, 0.0, 0.0) and g[2][3] == (1.0, 0.0, 0.0)
