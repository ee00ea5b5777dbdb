"""FFT schedule table and overrides (no GPU needed): the greedy default
orders, overrides through the C ABI, rejection of invalid radix lists, the
table file the autotuner writes (read through QDG_FFT_SCHEDULES in a fresh
process), and the autotuner's candidate generator."""
import ctypes as C
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from qdng_gb300 import _lib, build
    build.build()
    return _lib.load()


def _get(lib, ctx, n, prec):
    r = (C.c_int32 * 16)()
    ns, ln = C.c_int32(), C.c_int32()
    assert lib.qdg_fft_schedule_get(ctx, n, prec, r, C.byref(ns), C.byref(ln)) == 0
    return list(r)[:ns.value], ln.value


def test_greedy_defaults_and_overrides(lib):
    lib.qdg_fft_schedule_reset(0)  # the table off: greedy orders
    assert _get(lib, 0, 256, 0) == ([16, 16], 0)
    assert _get(lib, 0, 1024, 0) == ([16, 16, 4], 0)
    assert _get(lib, 1, 384, 1) == ([16, 8, 3], 0)
    arr = (C.c_int32 * 3)(4, 4, 16)
    assert lib.qdg_fft_schedule_set(0, 256, 0, arr, 3, 8) == 0
    assert _get(lib, 0, 256, 0) == ([4, 4, 16], 8)
    assert _get(lib, 0, 256, 1) == ([16, 16], 0)  # another precision is untouched
    assert lib.qdg_fft_schedule_set(0, 256, 0, (C.c_int32 * 2)(4, 32), 2, 0) != 0  # 32 is no radix
    assert lib.qdg_fft_schedule_set(0, 256, 0, (C.c_int32 * 2)(4, 16), 2, 0) != 0  # product 64
    assert lib.qdg_fft_schedule_set(0, 256, 0, arr, 3, 99) != 0                    # lines above 64
    lib.qdg_fft_schedule_reset(0)
    assert _get(lib, 0, 256, 0) == ([16, 16], 0)
    # with the table: the committed autotuner entry for this size, if any
    lib.qdg_fft_schedule_reset(1)
    want = ([16, 16], 0)
    for line in open(os.path.join(ROOT, "qdng_gb300", "fft_schedules.txt")):
        f = line.split("#")[0].split()
        if f[:3] == ["plan", "256", "fp64"]:
            want = ([int(x) for x in f[3].split(",")], int(f[4]))
    assert _get(lib, 0, 256, 0) == want


def test_table_file_is_read(tmp_path):
    t = tmp_path / "sched.txt"
    t.write_text("# comment\nplan 256 fp64 8,8,4 6   # tuned\nensemble 1024 mixed 4,16,16 0\n"
                 "plan 128 fp64 4,4,4 0\n")  # the last line is invalid (product 64) and skipped
    code = ("import ctypes as C\nfrom qdng_gb300 import _lib\nL=_lib.load()\n"
            "def g(c,n,p):\n r=(C.c_int32*16)(); ns=C.c_int32(); ln=C.c_int32()\n"
            " L.qdg_fft_schedule_get(c,n,p,r,C.byref(ns),C.byref(ln)); return list(r)[:ns.value], ln.value\n"
            "print(g(0,256,0), g(1,1024,1), g(0,128,0))\n")
    env = dict(os.environ, QDG_FFT_SCHEDULES=str(t))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "([8, 8, 4], 6) ([4, 16, 16], 0) ([16, 8], 0)"


def test_candidate_orders():
    from qdng_gb300.autotune import greedy, orders
    for n in (64, 96, 128, 256, 384, 1024, 3072, 4096):
        cands = orders(n)
        assert cands
        for c in cands:
            p = 1
            for r in c:
                p *= r
            assert p == n
        g = greedy(n)
        p = 1
        for r in g:
            p *= r
        assert p == n
    assert greedy(256) == [16, 16] and greedy(96) == [16, 2, 3] and greedy(1024) == [16, 16, 4]
