"""ctypes binding of oracle/_ref/libx2dhf_refc.so: the reference's own C
relaxation kernels (x2dhf src/c, built unmodified by oracle/build_ref.sh)
behind oracle/ref_shim.c.  TEST INFRASTRUCTURE ONLY."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libx2dhf_refc.so")
_lib = None


def available():
    if not os.path.exists(LIB):
        subprocess.call(["bash", os.path.join(HERE, "build_ref.sh")], stdout=subprocess.DEVNULL)
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference C kernels not built (oracle/build_ref.sh)")
        L = C.CDLL(LIB)
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        I = C.c_int
        L.x2r_setup.restype = I
        L.x2r_setup.argtypes = [I, I, ip, ip, I, ip, I, ip, I, ip, I, dp, dp, dp, dp, dp, dp, I]
        L.x2r_use_colour_lists.argtypes = [I]
        L.x2r_set_omega.argtypes = [C.c_double]
        L.x2r_sorpt.argtypes = [I, dp, dp, dp]
        L.x2r_mcsor.argtypes = [I, I, dp, dp, dp]
        L.x2r_set_functions.argtypes = [dp, ip, I, dp]
        L.x2r_set_batch.argtypes = [I, I, ip, ip, ip, ip, ip]
        L.x2r_coulexch.argtypes = [I]
        _lib = L
    return _lib


class RefKernels:
    """The reference kernels bound to one oracle case's grid and tables."""

    def __init__(self, case, maxsor2=10):
        L = lib()
        i1, i2, i6a, i6b, i7 = case.lists()
        dmu1, dmu2, dni1, dni2, ex, _ = case.coeffs()
        self.suppl = np.concatenate([case.suppl(k) for k in range(14)])
        self.keep = (i1, i2, i6a, i6b, i7)
        rc = L.x2r_setup(case.nni, case.nmu, i1, i2, i1.size, i6a, i6a.size, i6b, i6b.size, i7, i7.size,
                         dmu1, dmu2, dni1, dni2, ex, self.suppl, maxsor2)
        assert rc == 0
        self.L = L

    def sorpt(self, isym, omega, uext, lhs, rhs, colour_order=False):
        u = np.ascontiguousarray(uext, np.float64).copy()
        self.L.x2r_use_colour_lists(1 if colour_order else 0)
        self.L.x2r_set_omega(omega)
        self.L.x2r_sorpt(isym, u, np.ascontiguousarray(lhs), np.ascontiguousarray(rhs))
        return u

    def mcsor(self, isym, nthreads, omega, uext, lhs, rhs):
        u = np.ascontiguousarray(uext, np.float64).copy()
        self.L.x2r_set_omega(omega)
        self.L.x2r_mcsor(isym, nthreads, u, np.ascontiguousarray(lhs), np.ascontiguousarray(rhs))
        return u


POT_HOOK = C.CFUNCTYPE(None, C.c_void_p, C.c_int)
ORB_HOOK = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)


class ReferenceSCF:
    """The oracle's SCF driver with every relaxation done by the reference's
    own C backend: coulExch_pthread_ (one thread per potential, sorpt_ on the
    colour-ordered lists of a PT build with the mcsor card) and
    mcsor_pthread_ with `nthreads` threads for the orbitals."""

    def __init__(self, deck, nthreads=1):
        from oracle.pyoracle import Case, lib as olib

        self.case = Case(deck)
        self.rk = RefKernels(self.case)
        L, O = self.rk.L, olib()
        O.x2o_orbital_block.restype = C.c_void_p
        O.x2o_orbital_block.argtypes = [C.c_void_p]
        O.x2o_potential_block.restype = C.c_void_p
        O.x2o_potential_block.argtypes = [C.c_void_p]
        O.x2o_pot_offset.restype = C.c_long
        O.x2o_pot_offset.argtypes = [C.c_void_p, C.c_int, C.c_int]
        O.x2o_set_hooks.argtypes = [C.c_void_p, POT_HOOK, ORB_HOOK, C.c_void_p]
        h = self.case.h
        norb, mx = self.case.norb, self.case.mxsize
        set_functions = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p)(("x2r_set_functions", L))
        self.i1b = np.array([1 + i * mx for i in range(norb)], np.int32)
        set_functions(O.x2o_orbital_block(h), self.i1b.ctypes.data, norb, O.x2o_potential_block(h))
        self.batches = []
        for iorb in range(1, norb + 1):
            n = self.case.npots(iorb)
            info = [self.case.pot_info(iorb, k) for k in range(1, n + 1)]
            arr = [np.array(v, np.int32) for v in zip(*info)]
            ib = np.array([O.x2o_pot_offset(h, iorb, k) for k in range(1, n + 1)], np.int32)
            L.x2r_set_batch(iorb, n, arr[0], arr[1], ib, arr[2], arr[3])
            self.batches.append(arr + [ib])
        oo, op = self.case.omega()
        # the orbital hook passes raw pointers: a separately typed handle of
        # x2r_mcsor, leaving RefKernels' array-typed one untouched
        mcsor_vp = C.CFUNCTYPE(None, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)(("x2r_mcsor", L))

        def pot(ud, iorb):
            L.x2r_use_colour_lists(1)
            L.x2r_set_omega(op)
            L.x2r_coulexch(iorb)

        def orb(ud, iorb, isym, wk2, lhs, rhs):
            L.x2r_set_omega(oo)
            mcsor_vp(isym, nthreads, wk2, lhs, rhs)

        self._pot, self._orb = POT_HOOK(pot), ORB_HOOK(orb)
        O.x2o_set_hooks(h, self._pot, self._orb, None)

    def steps(self, n):
        return self.case.steps(n)

    def records(self):
        return self.case.records()
