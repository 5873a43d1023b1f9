"""x2dhf_gb300 -- GB300 (sm_103a) relaxation path of x2dhf.

Python host mirror of the reference's operator surface over the C ABI of
libx2dhf_gpu.so (include/x2dhf_gpu.h):

    parse_deck(text)        input cards -> x2g_case (src/inputInterface.F90)
    Context(device)         one GPU, one stream
    Grid(ctx, ...)          grid, operator tables, sweep schedule
    relax(ctx, grid, jobs)  batched (MC)SOR relaxation of device arrays
    SCF(ctx, case)          device-resident closed-shell HF SCF (src/doSCF.F90)

The library must be built (x2dhf_gb300.build.build()); there is no CPU
fallback: every call here runs the CUDA kernels or raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libx2dhf_gpu.so")

MAXORB = 36
FP64, MIXED, SOR = 0, 1, 2
_ERRORS = {1: "bad argument", 2: "CUDA error", 3: "allocation failed", 4: "device barrier timeout",
           5: "NaN detected", 6: "schedule check failed", 7: "COMMON blocks not linked",
           8: "unsupported case", 9: "no CUDA device"}


class X2GError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"x2g error {code} ({_ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Case(C.Structure):
    _fields_ = [
        ("z1", C.c_double), ("z2", C.c_double), ("r", C.c_double),
        ("nnu", C.c_int), ("nmu", C.c_int), ("rinf", C.c_double),
        ("norb", C.c_int), ("m", C.c_int * MAXORB), ("gu", C.c_byte * MAXORB), ("occ", C.c_double * MAXORB),
        ("co1", C.c_double * MAXORB), ("co2", C.c_double * MAXORB),
        ("za", C.c_double * MAXORB), ("zb", C.c_double * MAXORB),
        ("n1", C.c_int * MAXORB), ("l1", C.c_int * MAXORB), ("n2", C.c_int * MAXORB), ("l2", C.c_int * MAXORB),
        ("maxscf", C.c_int), ("ienterm", C.c_int), ("inoterm", C.c_int), ("ienterm4init", C.c_int),
        ("nscf2skip", C.c_int), ("nenlast", C.c_int), ("nnolast", C.c_int),
        ("maxsor_orb", C.c_int), ("maxsor_pot", C.c_int),
        ("omega_orb", C.c_double), ("omega_pot", C.c_double), ("recalc_mm", C.c_double),
        ("mpole", C.c_int), ("homonuclear", C.c_int), ("precision", C.c_int), ("start", C.c_int),
        ("orb_scheme", C.c_int), ("pot_scheme", C.c_int), ("batch_mode", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("iterations", C.c_int), ("converged", C.c_int), ("sweeps", C.c_long),
        ("total_energy", C.c_double), ("electronic_energy", C.c_double), ("virial", C.c_double),
        ("ee", C.c_double * MAXORB), ("norm_error", C.c_double * MAXORB),
    ]


class Job(C.Structure):
    _fields_ = [
        ("u", C.c_void_p), ("lhs", C.c_void_p), ("rhs", C.c_void_p), ("psa", C.c_void_p), ("psb", C.c_void_p),
        ("omega", C.c_double), ("isym", C.c_int), ("idel", C.c_int), ("kind", C.c_int), ("pad", C.c_int),
    ]


EXPORTS = [
    "x2g_last_status", "x2g_last_error", "x2g_create", "x2g_destroy", "x2g_synchronize", "x2g_stream",
    "x2g_grid_create", "x2g_grid_destroy", "x2g_round_grid", "x2g_nmu_from_rinf", "x2g_default_omega",
    "x2g_grid_table", "x2g_grid_info", "x2g_relax", "x2g_putin", "x2g_putout", "x2g_mcsor_host",
    "x2g_quadrature", "x2g_case_defaults", "x2g_scf_create", "x2g_scf_destroy", "x2g_scf_run",
    "x2g_scf_get_orbital", "x2g_scf_get_coulomb", "x2g_scf_nrecords", "x2g_scf_record",
    "x2g_scf_set_function", "x2g_scf_get_function", "x2g_scf_set_start_values", "x2g_scf_get_start_values",
    "x2g_kernel_launches", "x2g_transfer_bytes", "mcsor_pthread_", "mcsor_tpool_", "coulExch_pthread_", "coulExch_tpool_",
    "tpoolStop4mcsor_", "tpoolStop4pots_", "x2g_host_table", "x2g_host_schedule", "x2g_profile",
    "x2g_relax_noalloc", "x2g_host_cluster_plan", "x2g_set_mixed_on_chip", "x2g_set_potential_clusters", "x2g_cluster_occupancy",
    "x2g_set_mixed_colouring", "x2g_set_residual_overlap", "x2g_set_gram_orthonormalise",
    "x2g_host_cluster_chunks", "x2g_host_free_chunks", "x2g_host_band_schedule",
    "x2g_convert_selftest", "x2g_set_wait_limit", "x2g_host_sor_schedule",
]

_lib = None


def lib():
    """Load libx2dhf_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError(f"{LIBPATH} missing: run x2dhf_gb300.build.build() (no CPU fallback exists)")
    L = C.CDLL(LIBPATH)
    P, I, D = C.c_void_p, C.c_int, C.c_double
    PP = C.POINTER(C.c_void_p)
    dp = C.POINTER(C.c_double)
    L.x2g_last_status.restype = I
    L.x2g_last_error.restype = C.c_char_p
    L.x2g_create.argtypes = [PP, I]
    L.x2g_destroy.argtypes = [P]
    L.x2g_synchronize.argtypes = [P]
    L.x2g_stream.restype = P
    L.x2g_stream.argtypes = [P]
    L.x2g_grid_create.argtypes = [P, I, I, D, D, D, D, I, PP]
    L.x2g_grid_destroy.argtypes = [P]
    L.x2g_round_grid.argtypes = [I]
    L.x2g_nmu_from_rinf.argtypes = [I, D, D]
    L.x2g_default_omega.argtypes = [I, I, D, D, dp, dp]
    L.x2g_grid_table.argtypes = [P, I, dp]
    L.x2g_grid_info.argtypes = [P] + [C.POINTER(C.c_int)] * 5
    L.x2g_relax.argtypes = [P, P, C.POINTER(Job), I, I, I]
    L.x2g_relax_noalloc.argtypes = [P, P, C.POINTER(Job), I, I]
    L.x2g_convert_selftest.argtypes = [P, C.c_long, C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    L.x2g_putin.argtypes = [P, P, I, P, P]
    L.x2g_putout.argtypes = [P, P, P, P]
    L.x2g_mcsor_host.argtypes = [P, P, I, I, D, I, dp, dp, dp]
    L.x2g_quadrature.argtypes = [P, P, I, P, P, P, dp]
    L.x2g_case_defaults.argtypes = [C.POINTER(Case)]
    L.x2g_scf_create.argtypes = [P, C.POINTER(Case), PP]
    L.x2g_scf_destroy.argtypes = [P]
    L.x2g_scf_run.argtypes = [P, I, C.POINTER(Result)]
    L.x2g_scf_get_orbital.argtypes = [P, I, dp]
    L.x2g_scf_get_coulomb.argtypes = [P, I, dp]
    L.x2g_scf_set_function.argtypes = [P, I, I, I, I, dp]
    L.x2g_scf_get_function.argtypes = [P, I, I, I, I, dp]
    L.x2g_scf_set_start_values.argtypes = [P, dp, dp, dp, dp]
    L.x2g_scf_get_start_values.argtypes = [P, dp, dp, dp, dp]
    L.x2g_scf_nrecords.argtypes = [P]
    L.x2g_scf_record.argtypes = [P, I, C.POINTER(C.c_int), C.POINTER(C.c_int), dp, dp, dp]
    L.x2g_host_table.argtypes = [I, I, D, D, D, D, I, dp]
    ip = C.POINTER(C.c_int)
    L.x2g_host_schedule.argtypes = [I, I, ip, ip, ip, ip, ip, ip, ip]
    L.x2g_host_band_schedule.argtypes = [I, I, ip, ip, ip, ip, ip, ip, ip, ip]
    L.x2g_host_sor_schedule.argtypes = [I, I, ip, ip, ip, ip, ip, ip, ip, ip]
    L.x2g_profile.argtypes = [P, I, I, dp, dp, C.POINTER(C.c_long)]
    L.x2g_host_cluster_plan.argtypes = [I, I, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_long),
                                        C.POINTER(C.c_int)]
    L.x2g_set_mixed_on_chip.argtypes = [P, I]
    L.x2g_set_potential_clusters.argtypes = [P, I]
    L.x2g_set_mixed_colouring.argtypes = [P, I]
    L.x2g_set_residual_overlap.argtypes = [P, I]
    L.x2g_set_gram_orthonormalise.argtypes = [P, I]
    L.x2g_cluster_occupancy.argtypes = [P, P, C.POINTER(I), C.POINTER(I)]
    L.x2g_set_wait_limit.argtypes = [P, D]
    L.x2g_kernel_launches.restype = C.c_long
    L.x2g_kernel_launches.argtypes = [P]
    L.x2g_transfer_bytes.argtypes = [P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        L = lib()
        raise X2GError(rc, L.x2g_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


# ---------------------------------------------------------------------------
# input cards (src/inputInterface.F90:681-818, HF subset)
# ---------------------------------------------------------------------------
def round_grid(n):
    """nnucalc/nmucalc rounding: n = 1 (mod 6) and n - 6 = 0 (mod 5), rounding down."""
    return lib().x2g_round_grid(int(n))


def parse_deck(text, precision=FP64, batch_mode=0):
    """Parse a reference input deck into an x2g_case (closed-shell HF).

    The relaxation schemes follow the deck's cards as in the reference: SOR
    unless mcsor / mcsor-o (orbitals) or mcsor-ce (potentials) is given.
    batch_mode: 0 the reference's relaxation order, 1 all potentials of an
    SCF iteration in one launch, 2 then all orbitals in one launch too
    (x2g_case.batch_mode)."""
    L = lib()
    c = Case()
    L.x2g_case_defaults(C.byref(c))
    c.precision = precision
    c.batch_mode = int(batch_mode)
    lines = [ln.split("!")[0].replace(",", " ").split() for ln in text.splitlines()]
    lines = [[t.lower() for t in ln] for ln in lines if ln]
    i = 0
    grid = None
    norb = 0
    hydrogen = False
    altsweeps = False

    def nums(tok):
        out = []
        for t in tok:
            try:
                out.append(float(t.replace("d", "e")))
            except ValueError:
                break
        return out

    while i < len(lines):
        ln = lines[i]
        lab = ln[0][:8]
        i += 1
        if lab == "nuclei":
            v = nums(ln[1:])
            c.z1, c.z2, c.r = v[0], v[1], v[2]
            if len(ln) > 4 and ln[4] == "angstrom":
                c.r = c.r / 0.52917721067121204
        elif lab == "method":
            if ln[1] != "hf":
                raise ValueError("only method hf is supported")
        elif lab == "config":
            while True:
                card = lines[i]
                i += 1
                nb = int(card[0])
                sym = card[1]
                mt = {"sigma": 0, "pi": 1, "delta": 2, "phi": 3}[sym]
                rest = card[2:]
                gu = " "
                if rest and rest[0] in ("g", "u"):
                    gu = rest[0]
                    c.homonuclear = 1
                    rest = rest[1:]
                spins = [t for t in rest if t != "end"]
                occ = 2.0 if mt == 0 else 4.0
                if spins and spins[0][0] in "+-.":
                    # explicit spin occupation (read_config): one electron per + or -
                    occ = float(sum(1 for t in spins[:4] if t in ("+", "-")))
                for _ in range(nb):
                    c.m[norb] = mt
                    c.gu[norb] = ord(gu)
                    c.occ[norb] = occ
                    norb += 1
                if "end" in rest:
                    break
            c.norb = norb
            for k in range(norb):
                c.co1[k] = 1.0 if c.z1 > 2.2e-16 else 0.0
                c.co2[k] = 1.0 if c.z2 > 2.2e-16 else 0.0
        elif lab == "grid":
            grid = ln[1:]
        elif lab == "orbpot":
            if ln[1] == "old":
                # functions, moments and Lagrange multipliers from a
                # checkpoint (SCF.load_checkpoint), no frozen phase
                c.start = 1
                c.ienterm4init = 0
                hydrogen = True
                continue
            if ln[1] != "hydrogen":
                raise ValueError("only orbpot hydrogen and orbpot old are supported")
            hydrogen = True
            v = nums(ln[2:])
            if v:
                c.ienterm4init = int(v[0])
        elif lab == "lcao":
            v = nums(ln[1:])
            inclorb = int(v[0]) if v else 1
            for k in range(norb):
                a = lines[i]
                i += 1
                c.co1[k], c.n1[k], c.l1[k], c.za[k] = float(a[0]), int(a[1]), int(a[2]), float(a[3])
                c.co2[k], c.n2[k], c.l2[k], c.zb[k] = float(a[4]), int(a[5]), int(a[6]), float(a[7])
                if inclorb == 2:
                    c.za[k] = c.z1 - c.za[k]
                    c.zb[k] = c.z2 - c.zb[k]
        elif lab == "scf":
            v = [int(x) for x in nums(ln[1:])]
            for name, x in zip(("maxscf", "saveScfData", "ienterm", "inoterm", "verbose"), v):
                if hasattr(c, name):
                    setattr(c, name, x)
        elif lab == "conv":
            v = [int(x) for x in nums(ln[1:])]
            for name, x in zip(("nscf2skip", "nenlast", "nnolast"), v):
                setattr(c, name, x)
        elif lab in ("mcsor", "mcsor-o"):
            # read_mcsor / read_mcsor_o (inputInterface.F90:1910-1990): MCSOR
            # for the orbitals; the mcsor card also puts the potentials back
            # on SOR (lpotmcsor=.false.)
            c.orb_scheme = 1
            if lab == "mcsor":
                c.pot_scheme = 0
            v = [int(x) for x in nums(ln[1:])]
            if len(v) > 1:
                c.maxsor_orb = v[1]
            if lab == "mcsor" and len(v) > 2:
                c.maxsor_pot = v[2]
        elif lab == "mcsor-ce":
            # read_mcsor_ce (inputInterface.F90:1992-2028): MCSOR for the potentials
            c.pot_scheme = 1
            v = [int(x) for x in nums(ln[1:])]
            if len(v) > 1:
                c.maxsor_pot = v[1]
        elif lab == "omega":
            v = nums(ln[1:])
            if v and abs(v[0]) > 0:
                c.omega_orb = v[0]
            if len(v) > 1 and abs(v[1]) > 0:
                c.omega_pot = v[1]
        elif lab == "multipol":
            v = nums(ln[1:])
            c.recalc_mm = v[0] if v and v[0] > 2.2e-16 else 1e15
            if len(v) > 1:
                c.mpole = int(v[1])
        elif lab == "altsweep":
            altsweeps = True
        elif lab == "stop":
            break
    if grid is None or norb == 0 or not hydrogen:
        raise ValueError("deck needs nuclei, config, grid, orbpot hydrogen and lcao cards")
    if altsweeps and (c.orb_scheme == 0 or c.pot_scheme == 0):
        # reversed list order for odd orbitals (isstep=-1): not scheduled on the GPU
        raise ValueError("altsweeps with list-order SOR is not supported")
    # lcao coefficients normalised |c1|+|c2| = 1 (read_lcao, read_stop)
    for k in range(norb):
        s = abs(c.co1[k]) + abs(c.co2[k])
        if s > 2.2e-16:
            c.co1[k] /= s
            c.co2[k] /= s
    g = nums(grid)
    c.nnu = round_grid(int(g[0]))
    if len(g) >= 3 and abs(g[2]) > 0:
        c.nmu = round_grid(int(round(g[1])))
        c.rinf = g[2]
    else:
        c.rinf = g[1]
        c.nmu = lib().x2g_nmu_from_rinf(c.nnu, c.r, c.rinf)
    return c


def host_table(nnu, nmu, r, rinf, z1, z2, which):
    """Operator table built by the library's host setup (no GPU needed)."""
    out = np.zeros(nnu * nmu)
    _check(lib().x2g_host_table(nnu, nmu, r, rinf, z1, z2, which, _dp(out)))
    return out


def host_schedule(nnu, nmu):
    """(order, tile, colour, level) of every scheduled interior point (no GPU needed)."""
    L = lib()
    n, t, l = C.c_int(), C.c_int(), C.c_int()
    _check(L.x2g_host_schedule(nnu, nmu, C.byref(n), C.byref(t), C.byref(l), None, None, None, None))
    arrs = [np.zeros(n.value, np.int32) for _ in range(4)]
    ip = [a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs]
    _check(L.x2g_host_schedule(nnu, nmu, C.byref(n), C.byref(t), C.byref(l), *ip))
    list_order = np.zeros(n.value, np.int32)
    _check(L.x2g_host_schedule(nnu, nmu, C.byref(n), C.byref(t), C.byref(l),
                               list_order.ctypes.data_as(C.POINTER(C.c_int)), None, None, None))
    return list_order, arrs[0], arrs[1], arrs[2], arrs[3]


def host_band_schedule(nnu, nmu):
    """(pts, off, rows, tile_row0, tile_row1, nlevels) of the persistent-band sweep (no GPU needed)."""
    L = lib()
    n, t, lv = C.c_int(), C.c_int(), C.c_int()
    _check(L.x2g_host_band_schedule(nnu, nmu, C.byref(n), C.byref(t), C.byref(lv), None, None, None, None, None))
    pts = np.zeros(n.value, np.int32)
    off = np.zeros(5 * lv.value * (t.value + 1), np.int32)
    rows = np.zeros(17, np.int32)
    r0, r1 = np.zeros(t.value, np.int32), np.zeros(t.value, np.int32)
    ip = [a.ctypes.data_as(C.POINTER(C.c_int)) for a in (pts, off, rows, r0, r1)]
    _check(L.x2g_host_band_schedule(nnu, nmu, C.byref(n), C.byref(t), C.byref(lv), *ip))
    return pts, off, rows, r0, r1, lv.value


def host_sor_schedule(nnu, nmu):
    """(pts, off, bpts, boff, delta) of the list-order SOR wavefront (no GPU needed)."""
    L = lib()
    n, nl, nb, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    _check(L.x2g_host_sor_schedule(nnu, nmu, C.byref(n), C.byref(nl), C.byref(nb), C.byref(d),
                                   None, None, None, None))
    pts, off = np.zeros(n.value, np.int32), np.zeros(nl.value + 1, np.int32)
    boff = np.zeros(nb.value + 1, np.int32)
    _check(L.x2g_host_sor_schedule(nnu, nmu, C.byref(n), C.byref(nl), C.byref(nb), C.byref(d),
                                   None, None, None, boff.ctypes.data_as(C.POINTER(C.c_int))))
    bpts = np.zeros(int(boff[-1]), np.int32)
    ip = [a.ctypes.data_as(C.POINTER(C.c_int)) for a in (pts, off, bpts, boff)]
    _check(L.x2g_host_sor_schedule(nnu, nmu, C.byref(n), C.byref(nl), C.byref(nb), C.byref(d), *ip))
    return pts, off, bpts, boff, d.value


def host_cluster_chunks(nnu, nmu, colouring="reference"):
    """(packed chunks, segment offsets) of the on-chip sweep (no GPU needed);
    colouring "free": the seam-free colouring's plan."""
    L = lib()
    f = L.x2g_host_free_chunks if colouring == "free" else L.x2g_host_cluster_chunks
    nc, no = C.c_int(), C.c_int()
    _check(f(nnu, nmu, C.byref(nc), C.byref(no), None, None))
    ch = np.zeros(nc.value, np.int32)
    off = np.zeros(no.value, np.int32)
    _check(f(nnu, nmu, C.byref(nc), C.byref(no), ch.ctypes.data_as(C.POINTER(C.c_int)),
             off.ctypes.data_as(C.POINTER(C.c_int))))
    return ch.view(np.uint32), off


def host_cluster_plan(nnu, nmu):
    """(CTAs per job, max band rows, shared bytes per CTA, band starts) of the on-chip sweep."""
    L = lib()
    c, m, sm = C.c_int(), C.c_int(), C.c_long()
    _check(L.x2g_host_cluster_plan(nnu, nmu, C.byref(c), C.byref(m), C.byref(sm), None))
    rows = (C.c_int * (c.value + 1))()
    if c.value:
        _check(L.x2g_host_cluster_plan(nnu, nmu, C.byref(c), C.byref(m), C.byref(sm), rows))
    return c.value, m.value, sm.value, list(rows)


# ---------------------------------------------------------------------------
# objects
# ---------------------------------------------------------------------------
class Context:
    def __init__(self, device=0):
        self.L = lib()
        h = C.c_void_p()
        _check(self.L.x2g_create(C.byref(h), device))
        self.h = h

    def synchronize(self):
        _check(self.L.x2g_synchronize(self.h))

    @property
    def launches(self):
        return self.L.x2g_kernel_launches(self.h)

    def transfer_bytes(self):
        """(host-to-device, device-to-host) bytes the library has copied on this context."""
        a, b = C.c_longlong(), C.c_longlong()
        _check(self.L.x2g_transfer_bytes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_wait_limit(self, seconds):
        """Longest device-side wait of a persistent sweep block before the
        launch reports X2G_ERR_TIMEOUT (default 2 s; 0 fails any wait)."""
        _check(self.L.x2g_set_wait_limit(self.h, float(seconds)))

    def set_mixed_on_chip(self, on):
        """Mixed-form sweep path: True cluster kernel, False persistent-band
        kernel, "auto" cluster kernel up to its co-resident clusters."""
        _check(self.L.x2g_set_mixed_on_chip(self.h, 2 if on == "auto" else (1 if on else 0)))

    def set_potential_clusters(self, mode):
        """Cluster sweep of potential batches: True the two-CTAs-per-SM
        variant (residual only on chip, omega/lhs from row and column terms),
        False the plain kernel, "auto" the variant for batches above the
        plain kernel's co-resident clusters."""
        _check(self.L.x2g_set_potential_clusters(self.h, 2 if mode == "auto" else (1 if mode else 0)))

    def set_mixed_colouring(self, colouring):
        """Colouring of the mixed form's cluster sweep: "reference" (the
        reference's list order mod 5, seams level by level) or "free"
        (colour (col - row) mod 5, no seams)."""
        if colouring not in ("reference", "free"):
            raise ValueError("colouring must be 'reference' or 'free'")
        _check(self.L.x2g_set_mixed_colouring(self.h, 1 if colouring == "free" else 0))

    def set_gram_orthonormalise(self, on):
        """Batch mode 2: the orthonormalisation of an iteration in rounds
        with the loop's own sums (False, the default: bit-identical to the
        orbital-by-orbital loop) or through the orbitals' Gram matrix (True:
        faster, equal in exact arithmetic)."""
        _check(self.L.x2g_set_gram_orthonormalise(self.h, 1 if on else 0))

    def set_residual_overlap(self, on):
        """Potential batches beyond one wave of clusters: the later jobs' FP64
        residual on the auxiliary stream under the first wave's sweep."""
        _check(self.L.x2g_set_residual_overlap(self.h, 1 if on else 0))

    def convert_selftest(self, n, seed=1):
        """Mismatches of the integer-pipe FP64<->FP32 conversions against the hardware ones."""
        bad = C.c_ulonglong()
        _check(self.L.x2g_convert_selftest(self.h, n, seed, C.byref(bad)))
        return bad.value

    def profile(self, enable=-1, precision=FP64):
        """Sweep-kernel CUDA-event timing: (ms, point_updates, launches)."""
        ms, pts, n = C.c_double(), C.c_double(), C.c_long()
        _check(self.L.x2g_profile(self.h, enable, precision, C.byref(ms), C.byref(pts), C.byref(n)))
        return ms.value, pts.value, n.value

    def close(self):
        if getattr(self, "h", None):
            self.L.x2g_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Grid:
    def __init__(self, ctx, nnu, nmu, r, rinf, z1=1.0, z2=1.0, mpole=4):
        self.ctx = ctx
        self.L = lib()
        h = C.c_void_p()
        _check(self.L.x2g_grid_create(ctx.h, nnu, nmu, r, rinf, z1, z2, mpole, C.byref(h)))
        self.h = h
        self.nnu, self.nmu = nnu, nmu

    def info(self):
        v = [C.c_int() for _ in range(5)]
        _check(self.L.x2g_grid_info(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("nnu", "nmu", "ntiles", "nlevels", "npoints"), [x.value for x in v]))

    def cluster_occupancy(self):
        """(plain, potentials' variant) co-resident clusters of the mixed
        form's cluster sweep for this grid on the context's device."""
        a, b = C.c_int(), C.c_int()
        _check(self.L.x2g_cluster_occupancy(self.ctx.h, self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def table(self, which):
        out = np.zeros(self.nnu * self.nmu)
        _check(self.L.x2g_grid_table(self.h, which, _dp(out)))
        return out

    def close(self):
        # a grid outliving its context is left to the process teardown
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.L.x2g_grid_destroy(self.h)
        self.h = None

    def __del__(self):
        self.close()


def relax(ctx, grid, jobs, nsweeps, precision=FP64):
    """Relax a list of Job structures (device pointers) in one launch."""
    arr = (Job * len(jobs))(*jobs)
    _check(lib().x2g_relax(ctx.h, grid.h, arr, len(jobs), nsweeps, precision))


def relax_noalloc(ctx, grid, jobs, nsweeps):
    """FP64 relaxation through the entry point that allocates no device memory
    (fixed 32 MiB library-resident scratch; returns when the kernel is done)."""
    arr = (Job * len(jobs))(*jobs)
    _check(lib().x2g_relax_noalloc(ctx.h, grid.h, arr, len(jobs), nsweeps))


def mcsor_host(ctx, grid, isym, kind, omega, nsweeps, wk2, lhs, rhs):
    """One relaxation call on host arrays (wk2 extended, relaxed in place)."""
    _check(lib().x2g_mcsor_host(ctx.h, grid.h, isym, kind, omega, nsweeps, _dp(wk2), _dp(lhs), _dp(rhs)))
    return wk2


class SCF:
    def __init__(self, ctx, case):
        self.ctx = ctx
        self.L = lib()
        h = C.c_void_p()
        _check(self.L.x2g_scf_create(ctx.h, C.byref(case), C.byref(h)))
        self.h = h
        self.case = case

    def run(self, max_iterations=1 << 30):
        res = Result()
        _check(self.L.x2g_scf_run(self.h, max_iterations, C.byref(res)))
        return res

    def records(self):
        n = self.L.x2g_scf_nrecords(self.h)
        out = []
        a, b = C.c_int(), C.c_int()
        x, y, z = C.c_double(), C.c_double(), C.c_double()
        for i in range(n):
            _check(self.L.x2g_scf_record(self.h, i, C.byref(a), C.byref(b), C.byref(x), C.byref(y), C.byref(z)))
            out.append((a.value, b.value, x.value, y.value, z.value))
        return out

    def orbital(self, iorb):
        out = np.zeros(self.case.nnu * self.case.nmu)
        _check(self.L.x2g_scf_get_orbital(self.h, iorb, _dp(out)))
        return out

    def function(self, kind, i1, i2=0, which=0):
        """Plain nnu*nmu copy: kind 0 orbital, 1 Coulomb, 2 exchange (i1 <= i2)."""
        out = np.zeros(self.case.nnu * self.case.nmu)
        _check(self.L.x2g_scf_get_function(self.h, kind, i1, i2, which, _dp(out)))
        return out

    def load_checkpoint(self, ck):
        """orbpot old start from a checkpoint (x2dhf_gb300.checkpoint):
        orbitals, Coulomb and exchange potentials, Lagrange multipliers,
        norms and multipole moments, before the first run."""
        from .checkpoint import MAXMPOLE, MAXORB

        if (ck.nnu, ck.nmu, ck.norb) != (self.case.nnu, self.case.nmu, self.case.norb):
            raise ValueError("checkpoint grid or orbital count differs from the case")
        for i in range(1, ck.norb + 1):
            _check(self.L.x2g_scf_set_function(self.h, 0, i, 0, 0, _dp(np.ascontiguousarray(ck.orbitals[i - 1]))))
            _check(self.L.x2g_scf_set_function(self.h, 1, i, 0, 0, _dp(np.ascontiguousarray(ck.coulomb[i - 1]))))
        for (a, b, w), v in ck.exchange.items():
            _check(self.L.x2g_scf_set_function(self.h, 2, a, b, w, _dp(np.ascontiguousarray(v))))
        ee = np.ascontiguousarray(np.diag(ck.ee), np.float64)
        nrm = np.ones(ck.norb) if ck.orbnorm is None else np.ascontiguousarray(ck.orbnorm[:ck.norb], np.float64)
        cm = np.zeros(MAXORB * MAXMPOLE) if ck.cmulti is None else np.ascontiguousarray(ck.cmulti, np.float64)
        ex = (np.zeros(8 * MAXORB * (MAXORB + 1)) if ck.exc is None
              else np.ascontiguousarray(ck.exc, np.float64).reshape(-1))
        _check(self.L.x2g_scf_set_start_values(self.h, _dp(ee), _dp(nrm), _dp(cm), _dp(ex)))

    def checkpoint(self, title="x2dhf-gb300", nel=None):
        """The current state as a checkpoint (write it with checkpoint.write)."""
        from . import checkpoint as ckm

        c = self.case
        n, shape = c.norb, (c.nmu, c.nnu)
        m = [int(c.m[i]) for i in range(n)]
        ee, nrm = np.zeros(n), np.zeros(n)
        cm, ex = np.zeros(ckm.MAXORB * ckm.MAXMPOLE), np.zeros(8 * ckm.MAXORB * (ckm.MAXORB + 1))
        _check(self.L.x2g_scf_get_start_values(self.h, _dp(ee), _dp(nrm), _dp(cm), _dp(ex)))
        orbs = [self.function(0, i).reshape(shape) for i in range(1, n + 1)]
        couls = [self.function(1, i).reshape(shape) for i in range(1, n + 1)]
        exch = {k: self.function(2, *k).reshape(shape) for k in ckm.exchange_order(m)}
        nel = nel if nel is not None else int(round(sum(c.occ[i] for i in range(n))))
        return ckm.Checkpoint(title, c.nnu, c.nmu, c.rinf, c.z1, c.z2, c.r, nel, m, orbs, couls, exch, np.diag(ee),
                              nrm, cm, ex.reshape(8, -1))

    def coulomb(self, iorb):
        out = np.zeros(self.case.nnu * self.case.nmu)
        _check(self.L.x2g_scf_get_coulomb(self.h, iorb, _dp(out)))
        return out

    def close(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.L.x2g_scf_destroy(self.h)
        self.h = None

    def __del__(self):
        self.close()
