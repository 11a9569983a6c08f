"""Seeded synthetic tracker geometry and events for the segment-linking chain.

The reference library ships no geometry files and no events, so the workloads
are synthetic.  This module builds:

* a detector whose module ids follow the CMS outer-tracker detId layout that
  the reference decodes (``Module.h:27-44``, ``Module.cc:159-358``):
  barrel ``subdet<<25 | layer<<20 | side<<18 | rod<<10 | module<<2 | sensor``,
  endcap ``subdet<<25 | side<<23 | layer<<18 | ring<<12 | module<<2 | sensor``;
  the geometrically inner sensor of every pair is the one the reference calls
  "lower" (``Module.cc:229-232``, inversion rules ``Module.cc:239-302``);
* the three geometry tables in the reference's text formats
  (``TiltedGeometry.cc:18-41``: ``detId drdz slope``;
  ``EndcapGeometry.cc:18-61``: ``detId avgr2 yl sl yh sh c7 c8 cz`` with the
  centroid phi in column 7; ``ModuleConnectionMap.cc:18-47``:
  ``detId n d1 .. dn``), plus the same tables as arrays;
* events of helices in a 3.8 T field crossing the sensor planes, smeared,
  with uniform noise hits.

Everything is float64 numpy arithmetic rounded to float32 at the end, seeded by
``numpy.random.default_rng``; the arrays are bit-identical across x86-64 and
aarch64 hosts in practice, and :func:`fingerprint` lets a test confirm it.

Workloads (sizes as named by the benchmark configurations):

* ``barrel_flat``: 6 flat barrel layers, 100 helices pT log-uniform 1-10 GeV,
  |eta| < 0.8, 1,000 noise hits (about 2.2k hits);
* ``full``: barrel with layers 1-3 tilted for |z| > 20 cm, 5 disks per side;
  ``n_pu`` helices with pT = 0.6 + Exp(0.7) GeV plus 20 signal helices of
  2-50 GeV, |eta| < 2.5, 2 % noise (7,000 helices give about 150k hits).
"""
from __future__ import annotations

import hashlib
import math
import os
from dataclasses import dataclass, field

import numpy as np

# 1/R[cm] = KR / pT[GeV] for B = 3.8 T (the reference's kRinv1GeVf).
KR = 2.99792458e-3 * 3.8
SDL_INF = 123456789

BARREL_R = (21.8, 34.6, 49.9, 68.3, 87.8, 108.0)
BARREL_GAP = (0.26, 0.26, 0.26, 0.40, 0.40, 0.40)
ZMAX = 120.0
MOD_DZ = 5.0
FLAT_ZMAX_TILTED = 20.0
N_TILT_RINGS = int(round((ZMAX - FLAT_ZMAX_TILTED) / MOD_DZ))  # 20 per side
DISK_Z = (131.0, 156.0, 185.0, 220.0, 261.0)
DISK_NRINGS = (15, 15, 12, 12, 12)
EC_GAP = 0.4
EC_RMIN, EC_RMAX = 23.0, 110.0
LUM_Z = 15.0

KIND_FLAT, KIND_TILT, KIND_EC = 0, 1, 2


def barrel_detid(layer, side, rod, module, sensor):
    return ((5 << 25) | (layer << 20) | (side << 18) | (rod << 10)
            | (module << 2) | sensor)


def endcap_detid(side, layer, ring, module, sensor):
    return ((4 << 25) | (side << 23) | (layer << 18) | (ring << 12)
            | (module << 2) | sensor)


def is_inverted(subdet, side, layer, module):
    """Inversion parity rule of ``Module::parseIsInverted`` (Module.cc:239-302)."""
    if subdet == 4:
        return (module % 2 == 1) if side == 1 else (module % 2 == 0)
    if side == 3:
        return (module % 2 == 1) if layer <= 3 else (module % 2 == 0)
    return (module % 2 == 1) if layer <= 2 else (module % 2 == 0)


def sensor_bits(inverted):
    """(inner sensor bits, outer sensor bits): the inner sensor is 'lower'."""
    return (2, 1) if inverted else (1, 2)


@dataclass
class Detector:
    """All sensor modules as planes with in-plane bounds, plus the tables."""
    name: str
    # per sensor (both sensors of every pair), index = row
    detid: np.ndarray = None        # uint32
    kind: np.ndarray = None         # int8
    is_inner: np.ndarray = None     # bool (geometrically inner == reference 'lower')
    normal: np.ndarray = None       # (n,3) unit normal pointing away from the beam spot
    center: np.ndarray = None       # (n,3) point of the sensor plane at the module centre
    taxis: np.ndarray = None        # (n,3) in-plane tangential (r-phi) axis
    uaxis: np.ndarray = None        # (n,3) in-plane long axis (z / radial)
    half_t: np.ndarray = None       # tangential half width (barrel)
    half_z: np.ndarray = None       # half extent in z (barrel)
    r0: np.ndarray = None           # ring inner radius (endcap)
    r1: np.ndarray = None           # ring outer radius (endcap)
    phic: np.ndarray = None         # centre phi of the module
    dphi: np.ndarray = None         # half phi width (endcap)
    tilt: np.ndarray = None         # tilt angle in rz (tilted barrel)
    lower_index: dict = field(default_factory=dict)
    # tables
    tilted_rows: list = field(default_factory=list)   # (detid, drdz, slope)
    endcap_rows: list = field(default_factory=list)   # (detid, avgr2, yl, sl, yh, sh, c7, c8, cz)
    conn: dict = field(default_factory=dict)          # lower detid -> sorted list of lower detids
    has_tilt: bool = False
    has_endcap: bool = False

    # ------------------------------------------------------------------
    def n_phi(self, layer):
        return int(math.ceil(2.0 * math.pi * BARREL_R[layer - 1] / 10.0))

    def tables(self):
        """Geometry as arrays: (tilted, endcap, conn_detid, conn_off, conn_dst)."""
        tl = np.array(self.tilted_rows, dtype=np.float64).reshape(-1, 3)
        ec = np.array(self.endcap_rows, dtype=np.float64).reshape(-1, 9)
        keys = sorted(self.conn)
        off = np.zeros(len(keys) + 1, dtype=np.int64)
        dst = []
        for i, k in enumerate(keys):
            dst.extend(self.conn[k])
            off[i + 1] = len(dst)
        return (tl[:, 0].astype(np.uint32), tl[:, 1:].astype(np.float32),
                ec[:, 0].astype(np.uint32), ec[:, 1:].astype(np.float32),
                np.array(keys, dtype=np.uint32), off,
                np.array(dst, dtype=np.uint32))

    def write_files(self, outdir):
        """Write tilted/endcap/map text files in the reference's formats."""
        os.makedirs(outdir, exist_ok=True)
        paths = (os.path.join(outdir, "tilted_geometry.txt"),
                 os.path.join(outdir, "endcap_geometry.txt"),
                 os.path.join(outdir, "module_connection_map.txt"))
        with open(paths[0], "w") as f:
            for d, drdz, slope in self.tilted_rows:
                f.write("%d %.9g %.9g\n" % (d, np.float32(drdz), np.float32(slope)))
        with open(paths[1], "w") as f:
            for row in self.endcap_rows:
                f.write("%d " % row[0] + " ".join("%.9g" % np.float32(v) for v in row[1:]) + "\n")
        with open(paths[2], "w") as f:
            for k in sorted(self.conn):
                v = self.conn[k]
                f.write("%d %d" % (k, len(v)) + "".join(" %d" % d for d in v) + "\n")
        return paths

    def fingerprint(self):
        h = hashlib.sha256()
        for a in self.tables():
            h.update(np.ascontiguousarray(a).tobytes())
        return h.hexdigest()[:16]


# ----------------------------------------------------------------------
# detector construction
# ----------------------------------------------------------------------
def _slope_tangential(phi):
    """x-y slope of the module's tangential axis, with the reference's
    special values: SDL_INF for a module whose tangential axis is along y
    and exactly 0 when it is along x (MiniDoublet.cc:1084-1106)."""
    s, c = math.sin(phi), math.cos(phi)
    if abs(s) < 1e-12:
        return float(SDL_INF)
    if abs(c) < 1e-12:
        return 0.0
    return -c / s


def build_detector(kind: str = "full") -> Detector:
    """kind: 'barrel_flat' (6 flat barrel layers) or 'full' (tilted + endcap)."""
    tilted = kind == "full"
    endcap = kind == "full"
    rows = {k: [] for k in ("detid", "kind", "is_inner", "normal", "center", "taxis",
                            "uaxis", "half_t", "half_z", "r0", "r1", "phic", "dphi", "tilt")}

    def add(detid, kd, inner, n, c, t, u, ht=0.0, hz=0.0, r0=0.0, r1=0.0, pc=0.0, dp=0.0, tl=0.0):
        rows["detid"].append(detid); rows["kind"].append(kd); rows["is_inner"].append(inner)
        rows["normal"].append(n); rows["center"].append(c); rows["taxis"].append(t)
        rows["uaxis"].append(u); rows["half_t"].append(ht); rows["half_z"].append(hz)
        rows["r0"].append(r0); rows["r1"].append(r1); rows["phic"].append(pc)
        rows["dphi"].append(dp); rows["tilt"].append(tl)

    det = Detector(name=kind, has_tilt=tilted, has_endcap=endcap)
    for layer in range(1, 7):
        r = BARREL_R[layer - 1]
        gap = BARREL_GAP[layer - 1]
        nphi = det.n_phi(layer)
        ht = r * math.tan(math.pi / nphi)
        use_tilt = tilted and layer <= 3
        zlo = -FLAT_ZMAX_TILTED if use_tilt else -ZMAX
        nz = int(round(-2 * zlo / MOD_DZ))
        for k in range(1, nphi + 1):
            phi = 2.0 * math.pi * (k - 1) / nphi
            cp, sp = math.cos(phi), math.sin(phi)
            n = (cp, sp, 0.0)
            t = (-sp, cp, 0.0)
            # flat modules: rod = phi index, module = z index
            for iz in range(1, nz + 1):
                zc = zlo + MOD_DZ * (iz - 0.5)
                inv = is_inverted(5, 3, layer, iz)
                bi, bo = sensor_bits(inv)
                for bits, dr, inner in ((bi, 0.0, True), (bo, gap, False)):
                    c = ((r + dr) * cp, (r + dr) * sp, zc)
                    add(barrel_detid(layer, 3, k, iz, bits), KIND_FLAT, inner, n, c, t,
                        (0.0, 0.0, 1.0), ht=ht, hz=MOD_DZ / 2, pc=phi)
            if use_tilt:
                # tilted modules: rod = ring index along z, module = phi index
                for side in (1, 2):
                    sgn = 1.0 if side == 2 else -1.0
                    for ring in range(N_TILT_RINGS):
                        zabs = FLAT_ZMAX_TILTED + MOD_DZ * (ring + 0.5)
                        tilt = math.radians(25.0 + 35.0 * (zabs - FLAT_ZMAX_TILTED) / (ZMAX - FLAT_ZMAX_TILTED))
                        rod = ring + 1 if side == 2 else N_TILT_RINGS - ring
                        nt = (math.cos(tilt) * cp, math.cos(tilt) * sp, sgn * math.sin(tilt))
                        ut = (-math.sin(tilt) * cp, -math.sin(tilt) * sp, sgn * math.cos(tilt))
                        inv = is_inverted(5, side, layer, k)
                        bi, bo = sensor_bits(inv)
                        for bits, dr, inner in ((bi, 0.0, True), (bo, gap, False)):
                            c = (r * cp + dr * nt[0], r * sp + dr * nt[1], sgn * zabs + dr * nt[2])
                            d = barrel_detid(layer, side, rod, k, bits)
                            add(d, KIND_TILT, inner, nt, c, t, ut, ht=ht, hz=MOD_DZ / 2, pc=phi, tl=tilt)
                            det.tilted_rows.append((d, math.tan(tilt), _slope_tangential(phi)))
    if endcap:
        for side in (1, 2):
            sgn = 1.0 if side == 2 else -1.0
            for disk in range(1, 6):
                zd = DISK_Z[disk - 1]
                nr = DISK_NRINGS[disk - 1]
                dr_ring = (EC_RMAX - EC_RMIN) / nr
                for ring in range(1, nr + 1):
                    r0 = EC_RMIN + dr_ring * (ring - 1)
                    r1 = r0 + dr_ring
                    rm = 0.5 * (r0 + r1)
                    nmod = int(math.ceil(2.0 * math.pi * rm / 10.0))
                    for k in range(1, nmod + 1):
                        phi = 2.0 * math.pi * (k - 1) / nmod
                        cp, sp = math.cos(phi), math.sin(phi)
                        inv = is_inverted(4, side, disk, k)
                        bi, bo = sensor_bits(inv)
                        for bits, dz, inner in ((bi, 0.0, True), (bo, EC_GAP, False)):
                            z = sgn * (zd + dz)
                            d = endcap_detid(side, disk, ring, k, bits)
                            add(d, KIND_EC, inner, (0.0, 0.0, sgn), (rm * cp, rm * sp, z),
                                (-sp, cp, 0.0), (cp, sp, 0.0), r0=r0, r1=r1, pc=phi,
                                dp=math.pi / nmod)
                            sl = _slope_tangential(phi)
                            det.endcap_rows.append((d, rm * rm, 0.0, sl, 0.0, sl, phi, rm, z))
    for k, v in rows.items():
        arr = np.array(v)
        setattr(det, k, arr)
    det.detid = det.detid.astype(np.uint32)
    det.kind = det.kind.astype(np.int8)
    det.lower_index = {int(d): i for i, d in enumerate(det.detid) if det.is_inner[i]}
    det.conn = _module_map(det)
    return det


# ----------------------------------------------------------------------
# module lookups (lower sensors)
# ----------------------------------------------------------------------
def _barrel_lower_detid(det, layer, phi, z):
    """Vectorised: lower detid of the barrel module covering (phi, z) at layer,
    0 where none."""
    nphi = det.n_phi(layer)
    k = (np.floor(np.mod(phi, 2 * np.pi) / (2 * np.pi / nphi) + 0.5).astype(np.int64) % nphi) + 1
    out = np.zeros(phi.shape, dtype=np.uint32)
    use_tilt = det.has_tilt and layer <= 3
    zflat = FLAT_ZMAX_TILTED if use_tilt else ZMAX
    flat = np.abs(z) < zflat
    iz = np.floor((z + zflat) / MOD_DZ).astype(np.int64) + 1
    nz = int(round(2 * zflat / MOD_DZ))
    iz = np.clip(iz, 1, nz)
    inv = np.where(layer <= 3, iz % 2 == 1, iz % 2 == 0)
    bits = np.where(inv, 2, 1)
    ids = ((5 << 25) | (layer << 20) | (3 << 18) | (k << 10) | (iz << 2) | bits)
    out = np.where(flat, ids, out)
    if use_tilt:
        zabs = np.abs(z)
        ring = np.clip(np.floor((zabs - FLAT_ZMAX_TILTED) / MOD_DZ).astype(np.int64), 0, N_TILT_RINGS - 1)
        side = np.where(z > 0, 2, 1)
        rod = np.where(side == 2, ring + 1, N_TILT_RINGS - ring)
        inv = (k % 2 == 1) if layer <= 2 else (k % 2 == 0)
        bits = np.where(inv, 2, 1)
        ids = ((5 << 25) | (layer << 20) | (side << 18) | (rod << 10) | (k << 2) | bits)
        ok = (~flat) & (zabs <= ZMAX)
        out = np.where(ok, ids, out)
    out = np.where(np.abs(z) <= ZMAX, out, 0)
    return out.astype(np.uint32)


def _endcap_lower_detid(det, disk, side, rho, phi):
    nr = DISK_NRINGS[disk - 1]
    dr_ring = (EC_RMAX - EC_RMIN) / nr
    ring = np.floor((rho - EC_RMIN) / dr_ring).astype(np.int64) + 1
    ok = (rho >= EC_RMIN) & (rho < EC_RMAX)
    ring = np.clip(ring, 1, nr)
    rm = EC_RMIN + dr_ring * (ring - 0.5)
    nmod = np.ceil(2.0 * np.pi * rm / 10.0).astype(np.int64)
    k = (np.floor(np.mod(phi, 2 * np.pi) / (2 * np.pi / nmod) + 0.5).astype(np.int64) % nmod) + 1
    inv = np.where(side == 1, k % 2 == 1, k % 2 == 0)
    bits = np.where(inv, 2, 1)
    ids = ((4 << 25) | (side << 23) | (disk << 18) | (ring << 12) | (k << 2) | bits)
    return np.where(ok, ids, 0).astype(np.uint32)


def _module_map(det):
    """Lower module -> lower modules of the next layer that a straight line
    from the luminous region (|z0| <= 15 cm) through the module can reach,
    widened in phi by the bend of a 1 GeV track between the two radii."""
    idx = np.nonzero(det.is_inner)[0]
    z0s = np.array([-LUM_Z, -LUM_Z / 2, 0.0, LUM_Z / 2, LUM_Z])
    fr = np.array([-0.98, 0.0, 0.98])
    R1 = 1.0 / KR
    A, B = np.meshgrid(fr, fr, indexing="ij")
    A, B = A.ravel(), B.ravel()                       # 9 sample points
    ns = A.size
    src = np.repeat(idx, ns)
    a = np.tile(A, idx.size)
    b = np.tile(B, idx.size)
    kd = det.kind[src]
    hu = np.where(kd == KIND_TILT, det.half_z[src] / np.cos(det.tilt[src]), det.half_z[src])
    pb = det.center[src] + (a * det.half_t[src])[:, None] * det.taxis[src] + (b * hu)[:, None] * det.uaxis[src]
    rho_e = 0.5 * (det.r0[src] + det.r1[src]) + 0.5 * a * (det.r1[src] - det.r0[src])
    ph_e = det.phic[src] + b * det.dphi[src]
    pe = np.stack([rho_e * np.cos(ph_e), rho_e * np.sin(ph_e), det.center[src][:, 2]], axis=1)
    P = np.where((kd == KIND_EC)[:, None], pe, pb)
    nz = z0s.size
    src = np.repeat(src, nz)
    P = np.repeat(P, nz, axis=0)
    Z0 = np.tile(z0s, P.shape[0] // nz)
    d = det.detid[src].astype(np.int64)
    kd = det.kind[src]
    isec = kd == KIND_EC
    layer = np.where(isec, (d >> 18) & 7, (d >> 20) & 7)
    rhoP = np.hypot(P[:, 0], P[:, 1])
    phiP = np.arctan2(P[:, 1], P[:, 0])
    pairs_s, pairs_d = [], []

    def emit(mask, ids):
        ok = ids != 0
        pairs_s.append(det.detid[src[mask][ok]].astype(np.int64))
        pairs_d.append(ids[ok].astype(np.int64))

    def bend(rho):
        return np.abs(np.arcsin(np.minimum(rho / (2 * R1), 1)) - np.arcsin(np.minimum(rhoP / (2 * R1), 1)))

    for L in range(1, 6):
        m = (~isec) & (layer == L)
        if not np.any(m):
            continue
        rn = BARREL_R[L]
        zq = Z0 + (P[:, 2] - Z0) * (rn / rhoP)
        dphi = bend(np.full_like(rhoP, rn))
        inb = m & (np.abs(zq) <= ZMAX)
        for off in (-1.0, 0.0, 1.0):
            emit(inb, _barrel_lower_detid(det, L + 1, (phiP + off * dphi)[inb], zq[inb]))
        if det.has_endcap:
            out = m & (np.abs(zq) > ZMAX)
            side = np.where(zq > 0, 2, 1)
            zd = np.where(side == 2, DISK_Z[0], -DISK_Z[0])
            lamd = (zd - Z0) / (P[:, 2] - Z0)
            rho = rhoP * lamd
            dphi = bend(rho)
            okd = out & (lamd > 1)
            for off in (-1.0, 0.0, 1.0):
                emit(okd, _endcap_lower_detid(det, 1, side[okd], rho[okd], (phiP + off * dphi)[okd]))
    if det.has_endcap:
        for L in range(1, 5):
            m = isec & (layer == L)
            side = (d >> 23) & 3
            zn = np.where(side == 2, DISK_Z[L], -DISK_Z[L])
            lamd = (zn - Z0) / (P[:, 2] - Z0)
            rho = rhoP * lamd
            dphi = bend(rho)
            for off in (-1.0, 0.0, 1.0):
                emit(m, _endcap_lower_detid(det, L + 1, side[m], rho[m], (phiP + off * dphi)[m]))
    s = np.concatenate(pairs_s)
    t = np.concatenate(pairs_d)
    key = np.unique(s * (1 << 32) + t)
    s, t = key >> 32, key & 0xFFFFFFFF
    conn = {}
    bounds = np.nonzero(np.diff(s))[0] + 1
    for ss, tt in zip(np.split(s, bounds), np.split(t, bounds)):
        if ss.size:
            conn[int(ss[0])] = [int(v) for v in tt]
    return conn


# ----------------------------------------------------------------------
# events
# ----------------------------------------------------------------------
def _helix_point(tr, alpha):
    """Position on the helix after turning angle alpha (vectorised)."""
    R, h, phi0, cot, z0 = tr
    x = R * h * (np.sin(phi0 + h * alpha) - np.sin(phi0))
    y = -R * h * (np.cos(phi0 + h * alpha) - np.cos(phi0))
    z = z0 + R * alpha * cot
    return x, y, z


def _intersect_planes(tr, n, d, alpha0, iters=6):
    """Newton solve of n.p(alpha) = d starting at alpha0 (vectorised)."""
    R, h, phi0, cot, z0 = tr
    a = alpha0.copy()
    for _ in range(iters):
        x, y, z = _helix_point(tr, a)
        f = n[:, 0] * x + n[:, 1] * y + n[:, 2] * z - d
        dfx = R * np.cos(phi0 + h * a)
        dfy = R * np.sin(phi0 + h * a)
        dfz = R * cot
        fp = n[:, 0] * dfx + n[:, 1] * dfy + n[:, 2] * dfz
        fp = np.where(np.abs(fp) < 1e-12, 1e-12, fp)
        a = a - f / fp
    return a


def _plane_of(det, rows):
    n = det.normal[rows]
    c = det.center[rows]
    return n, np.einsum("ij,ij->i", n, c)


def _inside(det, rows, p):
    kd = det.kind[rows]
    rel = p - det.center[rows]
    tcoord = np.einsum("ij,ij->i", rel, det.taxis[rows])
    ok_b = (np.abs(tcoord) <= det.half_t[rows]) & (np.abs(rel[:, 2]) <= det.half_z[rows] + 1e-9)
    rho = np.hypot(p[:, 0], p[:, 1])
    ph = np.arctan2(p[:, 1], p[:, 0])
    dph = np.abs(np.mod(ph - det.phic[rows] + np.pi, 2 * np.pi) - np.pi)
    ok_e = (rho >= det.r0[rows]) & (rho < det.r1[rows]) & (dph <= det.dphi[rows] + 1e-12)
    return np.where(kd == KIND_EC, ok_e, ok_b)


def _rows_of(det, ids):
    """Sensor rows of detIds (vectorised; every id must exist)."""
    if not hasattr(det, "_order"):
        det._order = np.argsort(det.detid, kind="stable")
        det._sorted = det.detid[det._order]
    ids = np.asarray(ids, dtype=np.uint32)
    pos = np.searchsorted(det._sorted, ids)
    return det._order[pos]


def _partner_row(det, lower_rows):
    d = det.detid[lower_rows].astype(np.int64)
    part = np.where((d & 3) == 1, d + 1, d - 1)
    return _rows_of(det, part)


def _track_hits(det, tr, rng):
    """All sensor crossings of the helices in tr; returns (rows, points)."""
    R, h, phi0, cot, z0 = tr
    rows_all, pts_all = [], []
    # barrel layers
    for layer, branch in [(L, b) for L in range(1, 7) for b in (0, 1)]:
        # branch 0: outgoing crossing; branch 1: the looper's way back in
        r = BARREL_R[layer - 1]
        ok = r < 2 * R
        a_c = 2 * np.arcsin(np.minimum(r / (2 * R), 1.0))
        if branch:
            a_c = 2 * np.pi - a_c
        x, y, z = _helix_point(tr, a_c)
        ok &= np.abs(z) < ZMAX + 6
        trk = np.nonzero(ok)[0]
        if trk.size == 0:
            continue
        phi = np.arctan2(y[trk], x[trk])
        zt = z[trk]
        nphi = det.n_phi(layer)
        cand_ids = []
        for dk in (-1, 0, 1):
            for dzc in (-MOD_DZ, 0.0, MOD_DZ):
                ids = _barrel_lower_detid(det, layer, phi + dk * 2 * np.pi / nphi, zt + dzc)
                cand_ids.append(ids)
        cand_ids = np.stack(cand_ids, axis=1)  # (ntrk_sel, 9)
        best_a = {0: np.full(trk.size, np.inf), 1: np.full(trk.size, np.inf)}
        best_row = {0: np.full(trk.size, -1), 1: np.full(trk.size, -1)}
        best_p = {0: np.zeros((trk.size, 3)), 1: np.zeros((trk.size, 3))}
        for c in range(cand_ids.shape[1]):
            ids = cand_ids[:, c]
            valid = ids != 0
            if not np.any(valid):
                continue
            sel = np.nonzero(valid)[0]
            low_rows = _rows_of(det, ids[sel])
            up_rows = _partner_row(det, low_rows)
            sub = tuple(p[trk[sel]] for p in tr)
            for s, rows in ((0, low_rows), (1, up_rows)):
                n, dd = _plane_of(det, rows)
                a = _intersect_planes(sub, n, dd, a_c[trk[sel]])
                px, py, pz = _helix_point(sub, a)
                p = np.stack([px, py, pz], axis=1)
                lo, hi = (np.pi, 2 * np.pi) if branch else (0.0, np.pi)
                good = _inside(det, rows, p) & (a > lo) & (a < hi) & np.isfinite(a)
                better = good & (a < best_a[s][sel])
                idx = sel[better]
                best_a[s][idx] = a[better]
                best_row[s][idx] = rows[better]
                best_p[s][idx] = p[better]
        for s in (0, 1):
            m = best_row[s] >= 0
            rows_all.append(best_row[s][m])
            pts_all.append(best_p[s][m])
    # endcap disks
    if det.has_endcap:
        for disk in range(1, 6):
            for s in (0, 1):
                zabs = DISK_Z[disk - 1] + s * EC_GAP
                side = np.where(cot > 0, 2, 1)
                zs = np.where(side == 2, zabs, -zabs)
                with np.errstate(divide="ignore", invalid="ignore"):
                    a = (zs - z0) / (R * cot)
                ok = np.isfinite(a) & (a > 0) & (a < np.pi)
                trk = np.nonzero(ok)[0]
                if trk.size == 0:
                    continue
                sub = tuple(p[trk] for p in tr)
                px, py, pz = _helix_point(sub, a[trk])
                rho = np.hypot(px, py)
                ph = np.arctan2(py, px)
                ids = _endcap_lower_detid(det, disk, side[trk], rho, ph)
                good = ids != 0
                if not np.any(good):
                    continue
                low_rows = _rows_of(det, ids[good])
                rows = low_rows if s == 0 else _partner_row(det, low_rows)
                p = np.stack([px[good], py[good], pz[good]], axis=1)
                rows_all.append(rows)
                pts_all.append(p)
    rows = np.concatenate(rows_all) if rows_all else np.zeros(0, dtype=np.int64)
    pts = np.concatenate(pts_all) if pts_all else np.zeros((0, 3))
    return rows, pts


def _smear(det, rows, pts, rng):
    kd = det.kind[rows]
    ta = det.taxis[rows].copy()
    ua = det.uaxis[rows].copy()
    ec = kd == KIND_EC
    if np.any(ec):
        ph = np.arctan2(pts[ec, 1], pts[ec, 0])
        ta[ec] = np.stack([-np.sin(ph), np.cos(ph), np.zeros_like(ph)], axis=1)
        ua[ec] = np.stack([np.cos(ph), np.sin(ph), np.zeros_like(ph)], axis=1)
    st = rng.normal(0.0, 30e-4, size=len(rows))
    su = rng.normal(0.0, 0.05, size=len(rows))
    return pts + st[:, None] * ta + su[:, None] * ua


def _noise(det, n, rng):
    rows = rng.integers(0, len(det.detid), size=n)
    kd = det.kind[rows]
    a = rng.uniform(-1.0, 1.0, size=n)
    b = rng.uniform(-1.0, 1.0, size=n)
    hu = np.where(kd == KIND_TILT, det.half_z[rows] / np.cos(det.tilt[rows]), det.half_z[rows])
    pb = det.center[rows] + (a * det.half_t[rows])[:, None] * det.taxis[rows] + (b * hu)[:, None] * det.uaxis[rows]
    rho = np.sqrt(det.r0[rows] ** 2 + (b * 0.5 + 0.5) * (det.r1[rows] ** 2 - det.r0[rows] ** 2))
    ph = det.phic[rows] + a * det.dphi[rows]
    pe = np.stack([rho * np.cos(ph), rho * np.sin(ph), det.center[rows][:, 2]], axis=1)
    return rows, np.where((kd == KIND_EC)[:, None], pe, pb)


@dataclass
class Event:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    idx: np.ndarray
    detid: np.ndarray
    n_tracks: int = 0

    def __len__(self):
        return int(self.x.shape[0])

    def fingerprint(self):
        h = hashlib.sha256()
        for a in (self.x, self.y, self.z, self.idx, self.detid):
            h.update(np.ascontiguousarray(a).tobytes())
        return h.hexdigest()[:16]

    def write_bin(self, path):
        """Binary layout read by the oracle drivers: int64 n, then
        float32 x[n], y[n], z[n], int32 idx[n], uint32 detid[n]."""
        with open(path, "wb") as f:
            np.array([len(self)], dtype=np.int64).tofile(f)
            for a in (self.x, self.y, self.z, self.idx, self.detid):
                np.ascontiguousarray(a).tofile(f)


def make_event(det: Detector, seed: int, workload: str = "full", n_pu: int = 7000,
               n_signal: int = 20, noise_frac: float = 0.02) -> Event:
    """One seeded event.  workload 'barrel_flat' ignores n_pu/n_signal/noise_frac
    and makes 100 helices pT 1-10 GeV |eta| < 0.8 plus 1,000 noise hits."""
    rng = np.random.default_rng(seed)
    if workload == "barrel_flat":
        nt = 100
        pt = np.exp(rng.uniform(np.log(1.0), np.log(10.0), size=nt))
        eta = rng.uniform(-0.8, 0.8, size=nt)
    else:
        pt_pu = 0.6 + rng.exponential(0.7, size=n_pu)
        pt_sig = np.exp(rng.uniform(np.log(2.0), np.log(50.0), size=n_signal))
        pt = np.concatenate([pt_pu, pt_sig])
        nt = pt.size
        eta = rng.uniform(-2.5, 2.5, size=nt)
    phi0 = rng.uniform(-np.pi, np.pi, size=nt)
    z0 = rng.normal(0.0, 5.0, size=nt)
    q = np.where(rng.uniform(size=nt) < 0.5, -1.0, 1.0)
    R = pt / KR
    h = -q
    cot = np.sinh(eta)
    rows, pts = _track_hits(det, (R, h, phi0, cot, z0), rng)
    pts = _smear(det, rows, pts, rng)
    if workload == "barrel_flat":
        nn = 1000
    else:
        nn = int(round(noise_frac * len(rows)))
    nrows, npts = _noise(det, nn, rng)
    rows = np.concatenate([rows, nrows])
    pts = np.concatenate([pts, npts])
    perm = rng.permutation(len(rows))
    rows, pts = rows[perm], pts[perm]
    p32 = pts.astype(np.float32)
    n = len(rows)
    return Event(x=np.ascontiguousarray(p32[:, 0]), y=np.ascontiguousarray(p32[:, 1]),
                 z=np.ascontiguousarray(p32[:, 2]), idx=np.arange(n, dtype=np.int32),
                 detid=det.detid[rows].astype(np.uint32), n_tracks=nt)


_DET_CACHE = {}


def detector(kind: str = "full") -> Detector:
    if kind not in _DET_CACHE:
        _DET_CACHE[kind] = build_detector(kind)
    return _DET_CACHE[kind]


def workload_event(name: str, seed: int, pu: float = 200.0) -> tuple[Detector, Event]:
    """Named workloads: 'barrel_flat' (100 helices + 1k noise) or 'pu' (full
    geometry, pu/200 * 7,000 helices + 20 signal + 2 % noise)."""
    if name == "barrel_flat":
        det = detector("barrel_flat")
        return det, make_event(det, seed, "barrel_flat")
    det = detector("full")
    return det, make_event(det, seed, "full", n_pu=int(round(7000 * pu / 200.0)))
