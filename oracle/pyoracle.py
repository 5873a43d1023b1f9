"""ctypes binding of oracle/liboracle.so (TEST INFRASTRUCTURE ONLY).

The C restatement lives in oracle/x2dhf_oracle.c; see its header for the
reference file:line of every routine.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P, I, D = C.c_void_p, C.c_int, C.c_double
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.x2o_from_input.restype = P
        L.x2o_from_input.argtypes = [C.c_char_p, C.c_char_p, I]
        for n in ("x2o_setup", "x2o_nni", "x2o_nmu", "x2o_norb", "x2o_iterations", "x2o_nrecords"):
            getattr(L, n).restype = I
            getattr(L, n).argtypes = [P]
        L.x2o_run_scf.restype = I
        L.x2o_run_scf.argtypes = [P, I]
        L.x2o_scf_steps.restype = I
        L.x2o_scf_steps.argtypes = [P, I, I]
        L.x2o_free.argtypes = [P]
        for n in ("x2o_total_energy", "x2o_omega_orb", "x2o_omega_pot"):
            getattr(L, n).restype = D
            getattr(L, n).argtypes = [P]
        L.x2o_sweeps.restype = C.c_long
        L.x2o_sweeps.argtypes = [P]
        L.x2o_orbital_energy.restype = D
        L.x2o_orbital_energy.argtypes = [P, I]
        L.x2o_record.argtypes = [P, I] + [C.POINTER(C.c_int)] * 2 + [C.POINTER(C.c_double)] * 3
        L.x2o_ngrid.restype = I
        L.x2o_ngrid.argtypes = [P] + [C.POINTER(C.c_int)] * 4
        L.x2o_lists.argtypes = [P, ip, ip, ip, ip, ip]
        L.x2o_suppl.argtypes = [P, I, dp]
        L.x2o_coeffs.argtypes = [P, dp, dp, dp, dp, dp, C.POINTER(C.c_double)]
        L.x2o_get_orbital.argtypes = [P, I, dp]
        L.x2o_set_orbital.argtypes = [P, I, dp]
        L.x2o_npots.restype = I
        L.x2o_npots.argtypes = [P, I]
        L.x2o_pot_info.argtypes = [P, I, I] + [C.POINTER(C.c_int)] * 4
        L.x2o_get_pot.argtypes = [P, I, I, dp]
        L.x2o_set_pot.argtypes = [P, I, I, dp]
        L.x2o_set_orbital_energy.argtypes = [P, I, C.c_double]
        L.x2o_set_moments.argtypes = [P, dp, dp]
        L.x2o_putin.argtypes = [I, I, I, dp, dp]
        L.x2o_putout.argtypes = [I, I, dp, dp]
        L.x2o_sweep.argtypes = [P, I, I, I, D, dp, dp, dp, dp, dp, I, I, I]
        L.x2o_relax_pot.argtypes = [P, I, I, I]
        L.x2o_relax_orb.argtypes = [P, I, I]
        L.x2o_fock.argtypes = [P, I, dp, dp]
        L.x2o_norm_value.restype = D
        L.x2o_norm_value.argtypes = [P, I]
        L.x2o_norm.argtypes = [P, I]
        L.x2o_ortho.argtypes = [P, I]
        L.x2o_eahf.argtypes = [P, I]
        L.x2o_ee.restype = D
        L.x2o_ee.argtypes = [P, I, I]
        L.x2o_etotal.argtypes = [P] + [C.POINTER(C.c_double)] * 4
        L.x2o_mpole_moments.argtypes = [P, I]
        L.x2o_pot_asympt.argtypes = [P, I]
        L.x2o_cmulti.argtypes = [P, dp]
        L.x2o_set_batch_potentials.argtypes = [P, I]
        _lib = L
    return _lib


class Case:
    """One x2dhf case held by the oracle."""

    def __init__(self, deck: str, setup: bool = True):
        L = lib()
        err = C.create_string_buffer(256)
        self.h = L.x2o_from_input(deck.encode(), err, 256)
        if not self.h:
            raise ValueError(err.value.decode())
        self.L = L
        if setup:
            L.x2o_setup(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.x2o_free(self.h)
            self.h = None

    @property
    def nni(self):
        return self.L.x2o_nni(self.h)

    @property
    def nmu(self):
        return self.L.x2o_nmu(self.h)

    @property
    def norb(self):
        return self.L.x2o_norb(self.h)

    @property
    def mxsize(self):
        return self.nni * self.nmu

    def set_batch_potentials(self, mode=1):
        """1: all potentials of an SCF iteration relaxed from its starting
        orbitals; 2: then all orbitals from the state after them; 0: the
        reference's order."""
        self.L.x2o_set_batch_potentials(self.h, int(mode))

    def run(self, verbose=0):
        return self.L.x2o_run_scf(self.h, verbose)

    def steps(self, n, verbose=0):
        return bool(self.L.x2o_scf_steps(self.h, n, verbose))

    def records(self):
        out = []
        a, b = C.c_int(), C.c_int()
        x, y, z = C.c_double(), C.c_double(), C.c_double()
        for i in range(self.L.x2o_nrecords(self.h)):
            self.L.x2o_record(self.h, i, C.byref(a), C.byref(b), C.byref(x), C.byref(y), C.byref(z))
            out.append((a.value, b.value, x.value, y.value, z.value))
        return out

    def total_energy(self):
        return self.L.x2o_total_energy(self.h)

    def sweeps(self):
        return self.L.x2o_sweeps(self.h)

    def omega(self):
        return self.L.x2o_omega_orb(self.h), self.L.x2o_omega_pot(self.h)

    def lists(self):
        g = [C.c_int() for _ in range(4)]
        self.L.x2o_ngrid(self.h, *[C.byref(v) for v in g])
        n1, n6a, n6b, n7 = [v.value for v in g]
        a = [np.zeros(n, np.int32) for n in (n1, n1, n6a, n6b, n7)]
        self.L.x2o_lists(self.h, *a)
        return a

    def suppl(self, which):
        out = np.zeros(self.mxsize)
        self.L.x2o_suppl(self.h, which, out)
        return out

    def coeffs(self):
        a = [np.zeros(4) for _ in range(4)]
        ex = np.zeros(5)
        diag = C.c_double()
        self.L.x2o_coeffs(self.h, *a, ex, C.byref(diag))
        return a + [ex, diag.value]

    def orbital(self, iorb):
        out = np.zeros(self.mxsize)
        self.L.x2o_get_orbital(self.h, iorb, out)
        return out

    def set_orbital(self, iorb, v):
        self.L.x2o_set_orbital(self.h, iorb, np.ascontiguousarray(v, np.float64))

    def npots(self, iorb):
        return self.L.x2o_npots(self.h, iorb)

    def pot_info(self, iorb, k):
        v = [C.c_int() for _ in range(4)]
        self.L.x2o_pot_info(self.h, iorb, k, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)

    def pot(self, iorb, k):
        out = np.zeros(self.mxsize)
        self.L.x2o_get_pot(self.h, iorb, k, out)
        return out

    def set_pot(self, iorb, k, v):
        self.L.x2o_set_pot(self.h, iorb, k, np.ascontiguousarray(v, np.float64))

    def load_checkpoint(self, ck):
        """orbpot old: orbitals, Coulomb and exchange potentials and the
        diagonal Lagrange multipliers of a checkpoint (x2dhf_gb300.checkpoint)
        into the case's storage (readFuncs, src/diskInterface.F90:247-779)."""
        m = ck.m
        for i in range(1, ck.norb + 1):
            self.set_orbital(i, ck.orbitals[i - 1].reshape(-1))
            self.L.x2o_set_orbital_energy(self.h, i, float(ck.ee[i - 1, i - 1]))
        for iorb in range(1, ck.norb + 1):
            for k in range(1, self.npots(iorb) + 1):
                in1, in2, idel, _ = self.pot_info(iorb, k)
                if in1 == in2 and idel == 0:
                    v = ck.coulomb[in1 - 1]
                else:
                    a, b = min(in1, in2), max(in1, in2)
                    second = a != b and m[a - 1] > 0 and m[b - 1] > 0 and idel == m[a - 1] + m[b - 1]
                    v = ck.exchange[(a, b, 1 if second else 0)]
                self.set_pot(iorb, k, v.reshape(-1))
        self.L.x2o_set_moments(self.h, np.ascontiguousarray(ck.cmulti, np.float64),
                               np.ascontiguousarray(ck.exc, np.float64).reshape(-1))

    def relax_pot(self, iorb, k, mode=1):
        self.L.x2o_relax_pot(self.h, iorb, k, mode)

    def relax_orb(self, iorb, mode=1):
        self.L.x2o_relax_orb(self.h, iorb, mode)

    def putin(self, isym, fun):
        work = np.zeros((self.nni + 8) * (self.nmu + 8))
        self.L.x2o_putin(self.nni, self.nmu, isym, np.ascontiguousarray(fun, np.float64), work)
        return work

    def sweep(self, mode, isym, nsweeps, omega, uext, lhs, rhs, b, d):
        u = np.ascontiguousarray(uext, np.float64).copy()
        n1 = self.lists()[0].size
        self.L.x2o_sweep(self.h, mode, isym, nsweeps, omega, u, np.ascontiguousarray(lhs),
                         np.ascontiguousarray(rhs), np.ascontiguousarray(b), np.ascontiguousarray(d), 1, n1, 1)
        return u

    def fock(self, iorb):
        f1, f2 = np.zeros(self.mxsize), np.zeros(self.mxsize)
        self.L.x2o_fock(self.h, iorb, f1, f2)
        return f1, f2

    def ee(self, i, j):
        return self.L.x2o_ee(self.h, i, j)

    def etotal(self):
        v = [C.c_double() for _ in range(4)]
        self.L.x2o_etotal(self.h, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)


def with_hydrogen0(deck: str) -> str:
    """Emulate `orbpot hydrogen 0` (no frozen-orbital start)."""
    out = []
    for ln in deck.splitlines():
        if ln.strip().lower().startswith("orbpot"):
            ln = "orbpot hydrogen 0"
        out.append(ln)
    return "\n".join(out) + "\n"
