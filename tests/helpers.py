"""Case builders shared by the parity tests: seeded inputs, engines and
their oracle counterparts."""
import numpy as np

import so3g_gb300
from so3g_gb300 import synth
from so3g_gb300.proj import quat

DEG = np.pi / 180
SPINS = {1: "T", 2: "QU", 3: "TQU"}
COORDS = ["CAR", "CEA", "ARC", "SIN", "TAN", "ZEA", "Flat", "Quat"]
ZENITHAL = ("ARC", "SIN", "TAN", "ZEA")


def native_inputs(coord, n_det, n_time, seed):
    """Boresight and detector inputs in the native frame of `coord`."""
    rng = np.random.default_rng(seed)
    if coord == "Flat":
        t = np.linspace(0, 1, n_time)
        ang = rng.uniform(0, 2 * np.pi) + 3 * t
        bore = np.stack([40 * np.sin(7 * t) + rng.normal(0, .01, n_time),
                         25 * t + rng.normal(0, .01, n_time), np.cos(ang), np.sin(ang)], axis=1)
        g = rng.uniform(0, np.pi, n_det)
        dets = np.stack([rng.normal(0, 3, n_det), rng.normal(0, 3, n_det), np.cos(g),
                         np.sin(g)], axis=1)
        resp = np.stack([np.ones(n_det), rng.uniform(0.5, 1, n_det)], axis=1).astype(np.float32)
        return np.ascontiguousarray(bore), np.ascontiguousarray(dets), resp
    Q, dets, resp, gamma, _ = synth.workload(n_det, n_time, seed=seed, radius_deg=1.0,
                                             rate=50., throw=6., v_az=1.)
    resp = resp.copy()
    resp[:, 1] = rng.uniform(0.5, 1.0, n_det).astype(np.float32)
    el, az0 = 50., 180.
    if coord in ZENITHAL:
        # Native pole at the scan centre (lon=-az0, lat=el).
        q = (quat.euler(2, np.pi) * quat.euler(1, (el - 90) * DEG) * quat.euler(2, az0 * DEG))
    else:
        q = quat.euler(1, el * DEG) * quat.euler(2, az0 * DEG)
    qn = np.ascontiguousarray(np.asarray(q * quat.G3VectorQuat(Q)))
    return qn, np.ascontiguousarray(dets), resp


def flat_args(orc_coords, clip=0.85, npix=(48, 64)):
    """Pixelizor args (ny, nx, dy, dx, cry, crx) whose map covers ~clip of
    the samples' coordinate range."""
    x = orc_coords[..., 0].ravel()
    y = orc_coords[..., 1].ravel()
    ny, nx = npix
    xlo, xhi = np.percentile(x, [50 - 50 * clip, 50 + 50 * clip])
    ylo, yhi = np.percentile(y, [50 - 50 * clip, 50 + 50 * clip])
    dx = -(xhi - xlo) / nx          # negative, as RA increases to the left
    dy = (yhi - ylo) / ny
    crx = -xhi / dx + 1 - 0.5 + 0.37   # x=xhi lands near column 0
    cry = -ylo / dy + 1 - 0.5 + 0.21
    return (ny, nx, float(dy), float(dx), float(cry), float(crx))


def engine_name(coord, ncomp, tiled, bilinear):
    return "ProjEng_%s_%s_%s%s" % (coord, SPINS[ncomp], "Tiled" if tiled else "NonTiled",
                                   "_Bilinear" if bilinear else "")


class Case:
    """A ProjEng with seeded inputs."""

    def __init__(self, orc, coord="CAR", ncomp=3, tiled=False, bilinear=False, n_det=5,
                 n_time=4000, seed=1, tile_shape=(16, 20), active=None, hp=None):
        self.coord = coord
        self.ncomp = ncomp
        self.tiled = tiled
        self.bore, self.dets, self.resp = native_inputs(coord, n_det, n_time, seed)
        self.n_det, self.n_time = n_det, n_time
        rng = np.random.default_rng(seed + 100)
        self.signal = rng.standard_normal((n_det, n_time)).astype(np.float32)
        if hp is not None:
            nside, nest, nside_tile = hp
            name = "ProjEng_HP_%s_%s" % (SPINS[ncomp], "Tiled" if tiled else "NonTiled")
            args = (nside, int(nest), nside_tile, active)
            self.eng = getattr(so3g_gb300, name)(args)
            self.name, self.args = name, args
        else:
            probe = so3g_gb300.ProjEng_CAR_TQU_NonTiled((1, 1, 1., 1., 1., 1.))
            pz = probe._pz()
            pz.coord_sys = so3g_gb300._abi.COORD[coord]
            co = orc.coords(pz, self.bore, self.dets)
            args = flat_args(co)
            if tiled:
                args = args + tuple(tile_shape)
                if active is not None:
                    args = args + (active,)
            self.name = engine_name(coord, ncomp, tiled, bilinear)
            self.args = args
            self.eng = getattr(so3g_gb300, self.name)(args)
        self.pz = self.eng._pz()

    def all_tiles(self):
        return list(range(self.eng._n_tile()))

    def blank(self, lead, populate=None):
        """A zero map with leading shape `lead` (tiled: tiles in populate
        or all)."""
        e = self.eng
        if not self.tiled:
            return np.zeros(tuple(lead) + e._pix_shape())
        pop = set(self.all_tiles() if populate is None else populate)
        return [np.zeros(tuple(lead) + e._tile_pix_shape(i)) if i in pop else None
                for i in range(e._n_tile())]

    def random_map(self, lead, seed=7, populate=None):
        m = self.blank(lead, populate)
        rng = np.random.default_rng(seed)
        if isinstance(m, list):
            for t in m:
                if t is not None:
                    t[...] = rng.standard_normal(t.shape)
        else:
            m[...] = rng.standard_normal(m.shape)
        return m


def oracle_map(m):
    """(flat buffer, tile offsets) of a map for the oracle."""
    from oracle import pack_tiles
    if isinstance(m, list):
        return pack_tiles(m)
    return np.ascontiguousarray(m).ravel().copy(), None


def map_from_oracle(flat, offs, like):
    from oracle import unpack_tiles
    if offs is None:
        return flat.reshape(like.shape)
    return unpack_tiles(flat, offs, like)


def stack_map(m):
    if isinstance(m, list):
        return np.concatenate([t.ravel() for t in m if t is not None])
    return np.asarray(m).ravel()
