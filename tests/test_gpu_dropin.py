"""The reference-named drop-in symbols, called as a PTHREAD build of x2dhf
would call them.

libx2dhf_gpu.so exports mcsor_pthread_ and coulExch_pthread_ with the
signatures of src/c/mcsor_pthread.c:32 and src/c/coulExch_pthread.c:19 (the
Fortran bind(c) interfaces of src/relaxOrbs.F90:287-293 and
src/relaxPots.F90:147-151).  They read the Fortran COMMON blocks
(src/c/sorpt.h:58-249), which the library references weakly.  Here the
COMMON blocks come from oracle/_ref's shim, filled by x2r_setup exactly as
the Fortran program fills them, and the results are compared bit for bit
with the reference's own kernels built from its sources:

* mcsor_pthread_ on the GPU against the reference's mcsor_pthread_ on one
  thread (colour-reordered lists);
* coulExch_pthread_ on the GPU, every potential of an orbital in one launch,
  against the reference's sorpt_ on the colour-reordered lists;
* with the "middle" list in cw_sor (a build without the mcsor-ce card)
  coulExch_pthread_ runs list-order SOR on the GPU, against the reference's
  sorpt_ on the same list, instead of running MCSOR in its place.

Each case runs in a fresh process: the library's weak references bind when
it is loaded, so the COMMON blocks must be loaded before it.
"""
import json
import os
import subprocess
import sys

import pytest

from oracle import pyref

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not pyref.available(), reason="reference C sources not built")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r'''
import ctypes as C, json, sys
import numpy as np
sys.path.insert(0, ROOT); sys.path.insert(0, ROOT + "/tests")
from oracle import pyref
from oracle.pyoracle import Case, lib as olib
refc = C.CDLL(pyref.LIB, mode=C.RTLD_GLOBAL)          # COMMON blocks + the reference's kernels
import x2dhf_gb300 as xg
gpu = xg.lib()                                        # weak COMMON references bind to refc's blocks
from conftest import golden_deck
lines = [ln for ln in golden_deck(NAME).splitlines() if not ln.strip().lower().startswith("stop")]
deck = "\n".join(lines + ["mcsor", "mcsor-ce", "stop"]) + "\n"
oc = Case(deck)
rk = pyref.RefKernels(oc)
out = {}
dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
gpu.mcsor_pthread_.argtypes = [ip, ip, dp, dp, dp]
gpu.mcsor_pthread_.restype = None
gpu.coulExch_pthread_.argtypes = []
gpu.coulExch_pthread_.restype = None
def p(a):
    return a.ctypes.data_as(dp)
# --- mcsor_pthread_: an orbital relaxation call
iorb = 1
f1, f2 = oc.fock(iorb)
lhs, rhs = f1 + oc.coeffs()[5], f2.copy()
isym = -1 if xg.parse_deck(deck).m[iorb - 1] % 2 else 1   # pi orbitals are odd in nu
u = oc.putin(isym, oc.orbital(iorb))
omega = oc.omega()[0]
ref = rk.mcsor(isym, 1, omega, u, lhs, rhs)           # reference, 1 thread (sets omega, slices, colour lists)
wk2 = u.copy()
isym_c, nth = C.c_int(isym), C.c_int(4)
gpu.mcsor_pthread_(C.byref(isym_c), C.byref(nth), p(wk2), p(lhs), p(rhs))
out["mcsor_status"] = gpu.x2g_last_status()
out["mcsor_equal"] = bool(np.array_equal(wk2, ref))
out["mcsor_maxdiff"] = float(np.abs(wk2 - ref).max())
out["mcsor_changed"] = float(np.abs(ref - u).max())
# --- coulExch_pthread_: every potential of orbital IORB
O = olib()
O.x2o_orbital_block.restype = C.c_void_p; O.x2o_orbital_block.argtypes = [C.c_void_p]
O.x2o_potential_block.restype = C.c_void_p; O.x2o_potential_block.argtypes = [C.c_void_p]
O.x2o_pot_offset.restype = C.c_long; O.x2o_pot_offset.argtypes = [C.c_void_p, C.c_int, C.c_int]
norb, mx = oc.norb, oc.mxsize
L = rk.L
L.x2r_set_functions.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.int32), C.c_int, C.c_void_p]
i1b = np.array([1 + i * mx for i in range(norb)], np.int32)
L.x2r_set_functions(O.x2o_orbital_block(oc.h), i1b, norb, O.x2o_potential_block(oc.h))
for io in range(1, norb + 1):
    n = oc.npots(io)
    info = [oc.pot_info(io, k) for k in range(1, n + 1)]
    arr = [np.array(v, np.int32) for v in zip(*info)]
    ib = np.array([O.x2o_pot_offset(oc.h, io, k) for k in range(1, n + 1)], np.int32)
    L.x2r_set_batch(io, n, arr[0], arr[1], ib, arr[2], arr[3])
io = IORB
npots = oc.npots(io)
start = [oc.pot(io, k) for k in range(1, npots + 1)]
def restore():
    for k in range(1, npots + 1):
        oc.set_pot(io, k, start[k - 1])
L.x2r_set_omega(oc.omega()[1])
L.x2r_use_colour_lists(1)
L.x2r_coulexch(io)                                    # the reference's sorpt_, one thread per potential
refp = [oc.pot(io, k) for k in range(1, npots + 1)]
restore()
C.c_int.in_dll(refc, "c_interface_46_").value = io    # iorbc, as coulExchSORPT sets it
gpu.coulExch_pthread_()
out["coulexch_status"] = gpu.x2g_last_status()
got = [oc.pot(io, k) for k in range(1, npots + 1)]
out["npots"] = npots
out["coulexch_equal"] = all(bool(np.array_equal(a, b)) for a, b in zip(got, refp))
out["coulexch_maxdiff"] = max(float(np.abs(a - b).max()) for a, b in zip(got, refp))
out["coulexch_changed"] = max(float(np.abs(a - s).max()) for a, s in zip(refp, start))
# --- the middle list in cw_sor: list-order SOR, against the reference's sorpt_ on it
restore()
L.x2r_use_colour_lists(0)
L.x2r_coulexch(io)
refs = [oc.pot(io, k) for k in range(1, npots + 1)]
restore()
gpu.coulExch_pthread_()
out["sor_status"] = gpu.x2g_last_status()
got = [oc.pot(io, k) for k in range(1, npots + 1)]
out["sor_equal"] = all(bool(np.array_equal(a, b)) for a, b in zip(got, refs))
out["sor_maxdiff"] = max(float(np.abs(a - b).max()) for a, b in zip(got, refs))
out["sor_differs_from_mcsor"] = max(float(np.abs(a - b).max()) for a, b in zip(refs, refp))
print("RESULT " + json.dumps(out))
'''


def _run(name, iorb):
    code = DRIVER.replace("ROOT", repr(ROOT)).replace("NAME", repr(name)).replace("IORB", str(iorb))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    return json.loads(line[7:])


@pytest.mark.parametrize("name,iorb", [("ne_set01", 1), ("ne_set01", 4), ("h2_set01", 1)])
def test_reference_named_symbols_match_reference_kernels(name, iorb):
    out = _run(name, iorb)
    assert out["mcsor_status"] == 0 and out["mcsor_changed"] > 0
    assert out["mcsor_equal"], out["mcsor_maxdiff"]
    assert out["coulexch_status"] == 0 and out["npots"] >= 1 and out["coulexch_changed"] > 0
    assert out["coulexch_equal"], out["coulexch_maxdiff"]
    assert out["sor_status"] == 0 and out["sor_differs_from_mcsor"] > 0
    assert out["sor_equal"], out["sor_maxdiff"]
