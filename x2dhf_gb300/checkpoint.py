"""x2dhf checkpoint files: <prefix>.dat, .orb, .coul, .exch.

The reference writes them with writeToDisk / wtdisknat
(src/diskInterface.F90:1143-1213, src/dumpDataToDisk.F90:146-336) and reads
them for `orbpot old` with readFromDisk / readFuncs
(src/diskInterface.F90:1099-1136, 247-779).  Layout of the native form
(the default; 64-bit reals, 32-bit integers):

* .dat  text: title (75 characters); date and program version; `nnu nmu
  Rinf`; `Z1 Z2 R`; `norb nel nexch`.
* .orb  Fortran unformatted sequential records, each framed by its byte
  count (4-byte little-endian integer) before and after:
    1. the 15 address arrays i1b i2b i3b i1e i2e i3e i1si i2si i3si i1ng
       i2ng i3ng i1mu i2mu i3mu (int32; the i1/i2 arrays MAXORB long, the i3
       arrays MAXORB(MAXORB+1)/2), as set up by initAddr
       (src/initCBAllocArrays.F90:1147-1275);
    2. one record per orbital: nnu*nmu reals, nu fastest;
    3. orbNorm (MAXORB), ee (MAXORB x MAXORB, column-major), cmulti
       (MAXORB*MAXMPOLE), excdi, excqu, excoc, exche, exc5, exc6, exc7, exc8
       (MAXORB*(MAXORB+1) each).
* .coul one record per orbital's Coulomb potential.
* .exch the exchange potentials, for iorb1 <= iorb2 (a sigma orbital has no
  self-exchange potential): the potential of the pair, then for two
  non-sigma orbitals iorb1 < iorb2 the second one (Delta m = m1 + m2).

MAXORB = 36 and MAXMPOLE = 8 are the reference build's array dimensions;
they fix the record lengths.  Orbitals are numbered as in the reference
(the order of the config card).
"""
import dataclasses
import struct
import time

import numpy as np

MAXORB = 36
MAXMPOLE = 8
_NEXC = 8  # excdi, excqu, excoc, exche, exc5, exc6, exc7, exc8


@dataclasses.dataclass
class Checkpoint:
    title: str
    nnu: int
    nmu: int
    rinf: float
    z1: float
    z2: float
    r: float
    nel: int
    m: list                  # |lambda| of every orbital (0 sigma, 1 pi, ...)
    orbitals: list           # norb arrays (nmu, nnu)
    coulomb: list            # norb arrays (nmu, nnu)
    exchange: dict           # (iorb1, iorb2, which) -> (nmu, nnu), 1-based, iorb1 <= iorb2
    ee: np.ndarray           # Lagrange multipliers (norb, norb)
    orbnorm: np.ndarray = None
    cmulti: np.ndarray = None    # MAXORB*MAXMPOLE, as stored
    exc: np.ndarray = None       # (8, MAXORB*(MAXORB+1)), as stored
    date: str = ""
    version: str = ""
    nexch: int = None            # header count (initAddr's nexchpotsTot; 0 from the serial SOR path)
    ee_stored: np.ndarray = None  # the whole MAXORB x MAXORB record as read

    @property
    def norb(self):
        return len(self.m)


def exchange_order(m):
    """(iorb1, iorb2, which) of every exchange potential in file order."""
    out = []
    n = len(m)
    for i1 in range(1, n + 1):
        for i2 in range(i1, n + 1):
            if i1 == i2 and m[i1 - 1] == 0:
                continue
            out.append((i1, i2, 0))
            if i1 != i2 and m[i1 - 1] > 0 and m[i2 - 1] > 0:
                out.append((i1, i2, 1))
    return out


def _records(blob):
    recs, off = [], 0
    while off < len(blob):
        (n,) = struct.unpack_from("<i", blob, off)
        (n2,) = struct.unpack_from("<i", blob, off + 4 + n)
        if n != n2 or n < 0:
            raise ValueError(f"broken Fortran record at byte {off}")
        recs.append(blob[off + 4:off + 4 + n])
        off += n + 8
    return recs


def _record(data):
    b = data.tobytes()
    return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))


def address_arrays(norb, m, nnu, nmu):
    """initAddr's address arrays (src/initCBAllocArrays.F90:1172-1275) for
    one grid: orbitals and Coulomb potentials in consecutive nnu*nmu blocks,
    exchange potentials after (norb + 2) blocks, two blocks for a pair of
    non-sigma orbitals."""
    mx = nnu * nmu
    P = MAXORB * (MAXORB + 1) // 2
    a = {k: np.zeros(MAXORB, np.int32) for k in ("i1b", "i2b", "i1e", "i2e", "i1si", "i2si", "i1ng", "i2ng",
                                                  "i1mu", "i2mu")}
    a.update({k: np.zeros(P, np.int32) for k in ("i3b", "i3e", "i3si", "i3ng", "i3mu")})
    for i in range(norb):
        for p in ("1", "2"):
            a[f"i{p}b"][i] = i * mx + 1
            a[f"i{p}e"][i] = (i + 1) * mx
            a[f"i{p}si"][i] = mx
            a[f"i{p}ng"][i] = 1
            a[f"i{p}mu"][i] = nmu
    iend = (norb + 2) * mx
    for i1 in range(1, norb + 1):
        for i2 in range(i1, norb + 1):
            k = i1 + i2 * (i2 - 1) // 2 - 1
            if i1 == i2 and m[i1 - 1] == 0:
                continue
            iend += mx
            a["i3e"][k], a["i3b"][k], a["i3si"][k], a["i3ng"][k], a["i3mu"][k] = iend, iend - mx + 1, mx, 1, nmu
            if i1 != i2 and m[i1 - 1] > 0 and m[i2 - 1] > 0:
                iend += mx
    order = ("i1b", "i2b", "i3b", "i1e", "i2e", "i3e", "i1si", "i2si", "i3si", "i1ng", "i2ng", "i3ng", "i1mu",
             "i2mu", "i3mu")
    return np.concatenate([a[k] for k in order])


def read(prefix, m):
    """Read <prefix>.{dat,orb,coul,exch}; m = |lambda| of each orbital in the
    reference's order (the file does not store the symmetries)."""
    with open(prefix + ".dat") as f:
        lines = f.read().splitlines()
    title = lines[0].rstrip()
    date_version = lines[1]
    v = lines[2].split()
    nnu, nmu, rinf = int(v[0]), int(v[1]), float(v[2])
    v = lines[3].split()
    z1, z2, r = float(v[0]), float(v[1]), float(v[2])
    v = lines[4].split()
    norb, nel, nexch = int(v[0]), int(v[1]), int(v[2])
    if norb != len(m):
        raise ValueError(f"{prefix}.dat has {norb} orbitals, {len(m)} symmetries given")
    mx = nnu * nmu

    def arr(rec):
        if len(rec) != mx * 8:
            raise ValueError(f"record of {len(rec)} bytes, expected {mx * 8}")
        return np.frombuffer(rec, "<f8").reshape(nmu, nnu).copy()

    with open(prefix + ".orb", "rb") as f:
        recs = _records(f.read())
    if len(recs) != 1 + norb + 3 + _NEXC:
        raise ValueError(f"{prefix}.orb has {len(recs)} records, expected {1 + norb + 3 + _NEXC}")
    orbitals = [arr(recs[1 + i]) for i in range(norb)]
    extra = recs[1 + norb:]
    orbnorm = np.frombuffer(extra[0], "<f8").copy()
    ee_full = np.frombuffer(extra[1], "<f8").reshape(MAXORB, MAXORB, order="F")
    cmulti = np.frombuffer(extra[2], "<f8").copy()
    exc = np.stack([np.frombuffer(x, "<f8") for x in extra[3:]])
    with open(prefix + ".coul", "rb") as f:
        crecs = _records(f.read())
    if len(crecs) != norb:
        raise ValueError(f"{prefix}.coul has {len(crecs)} records, expected {norb}")
    coulomb = [arr(x) for x in crecs]
    order = exchange_order(m)
    with open(prefix + ".exch", "rb") as f:
        erecs = _records(f.read())
    if len(erecs) != len(order):
        raise ValueError(f"{prefix}.exch has {len(erecs)} records, expected {len(order)}")
    exchange = {key: arr(x) for key, x in zip(order, erecs)}
    return Checkpoint(title, nnu, nmu, rinf, z1, z2, r, nel, list(m), orbitals, coulomb, exchange,
                      ee_full[:norb, :norb].copy(), orbnorm.copy(), cmulti, exc,
                      date_version[:25], date_version[25:].strip(), nexch, ee_full.copy())


def fortran_e(x, w=25, d=16):
    """x as Fortran's Ew.d edit descriptor writes it: 0.<d digits>E+ee."""
    if x == 0.0:
        body = "0." + "0" * d + "E+00"
    else:
        mant, ex = f"{abs(x):.{d - 1}E}".split("E")
        digits = mant.replace(".", "")
        e = int(ex) + 1
        body = ("-" if x < 0 else "") + "0." + digits + ("E+" if e >= 0 else "E-") + f"{abs(e):02d}"
    return f"{body:>{w}}"


def write(prefix, ck, version="x2dhf-gb300"):
    """Write <prefix>.{dat,orb,coul,exch} in the reference's native form."""
    norb, mx = ck.norb, ck.nnu * ck.nmu
    nexch = ck.nexch if ck.nexch is not None else len(exchange_order(ck.m))
    date = time.strftime("%Y/%m/%d  %H:%M:%S.00 ")
    with open(prefix + ".dat", "w") as f:
        f.write(f"{ck.title[:75]:<75}\n")
        f.write(f"{date:<25}{version:<15}\n")
        f.write(f"{ck.nnu:5d}{ck.nmu:5d}{fortran_e(ck.rinf)}   / nnu nmu Rinf\n")
        f.write(f"{fortran_e(ck.z1)}{fortran_e(ck.z2)}{fortran_e(ck.r)}   / Z1 Z2 R\n")
        f.write(f"{norb:5d}{ck.nel:5d}{nexch:5d}    / norb nel nexch\n")

    def body(a):
        a = np.ascontiguousarray(a, dtype="<f8").reshape(-1)
        if a.size != mx:
            raise ValueError("function of the wrong size")
        return _record(a)

    orbnorm = np.zeros(MAXORB)
    if ck.orbnorm is not None:
        n = min(MAXORB, len(ck.orbnorm))
        orbnorm[:n] = ck.orbnorm[:n]
    ee = np.array(ck.ee_stored, dtype=np.float64) if ck.ee_stored is not None else np.zeros((MAXORB, MAXORB))
    ee[:norb, :norb] = ck.ee
    cmulti = ck.cmulti if ck.cmulti is not None else np.zeros(MAXORB * MAXMPOLE)
    exc = ck.exc if ck.exc is not None else np.zeros((_NEXC, MAXORB * (MAXORB + 1)))
    with open(prefix + ".orb", "wb") as f:
        f.write(_record(address_arrays(norb, ck.m, ck.nnu, ck.nmu).astype("<i4")))
        for o in ck.orbitals:
            f.write(body(o))
        f.write(_record(orbnorm.astype("<f8")))
        f.write(_record(np.asfortranarray(ee).T.reshape(-1).astype("<f8")))
        f.write(_record(np.asarray(cmulti, "<f8")))
        for x in exc:
            f.write(_record(np.asarray(x, "<f8")))
    with open(prefix + ".coul", "wb") as f:
        for c in ck.coulomb:
            f.write(body(c))
    with open(prefix + ".exch", "wb") as f:
        for key in exchange_order(ck.m):
            f.write(body(ck.exchange[key]))
