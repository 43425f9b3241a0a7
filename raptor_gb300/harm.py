"""HARM 2D ASCII dump and model.in I/O, in the formats the reference reads.

* Dump header: 26 whitespace-separated fields in the order of
  raptor_harm_model.c:90-115 (t n1 n2 startx1 startx2 dx1 dx2 tf nstep a gam
  cour DTd DTl DTi DTr dump_cnt image_cnt rdump_cnt dt lim failed Rin Rout
  hslope R0), then N1*N2 cell records, i outer / j inner
  (raptor_harm_model.c:147-149), each with 34 values: x1 x2 r h, the eight
  primitives rho u U1 U2 U3 B1 B2 B3, divb, ucon[4] ucov[4] bcon[4] bcov[4],
  vmin vmax vmin vmax, gdet (raptor_harm_model.c:150-169).
* model.in: eleven "NAME (unit) value" lines read positionally by
  read_model (core.c:22-34).

The reader is the host-side ingest for the engine: it fills the primitive
array [8][N1][N2] directly (no pointer-chased real****, grmhd.c:76-91) and
checks the header dimensions, which the reference does not enforce
(raptor_harm_model.c:116-119 calls `exit;` without parentheses).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from .synth import Dump, GridGeom

HEADER_INT_FIELDS = {"n1", "n2", "nstep", "DTr", "dump_cnt", "image_cnt", "rdump_cnt", "lim", "failed"}
HEADER_FIELDS = ("t", "n1", "n2", "startx1", "startx2", "dx1", "dx2", "tf", "nstep", "a", "gam",
                 "cour", "DTd", "DTl", "DTi", "DTr", "dump_cnt", "image_cnt", "rdump_cnt", "dt",
                 "lim", "failed", "Rin", "Rout", "hslope", "R0")
VALUES_PER_CELL = 34


class DumpFormatError(ValueError):
    pass


def write_dump(path: str | os.PathLike, dump: Dump) -> None:
    g = dump.geom
    ex = dump.extras
    hdr = dict(t=0.0, n1=g.n1, n2=g.n2, startx1=g.startx1, startx2=g.startx2, dx1=g.dx1,
               dx2=g.dx2, tf=2000.0, nstep=0, a=g.a, gam=g.gam, cour=0.9, DTd=5.0, DTl=0.5,
               DTi=1.0, DTr=1000, dump_cnt=0, image_cnt=0, rdump_cnt=0, dt=0.01, lim=0,
               failed=0, Rin=g.Rin, Rout=g.Rout, hslope=g.hslope, R0=g.R0)
    parts = []
    for k in HEADER_FIELDS:
        v = hdr[k]
        parts.append(str(int(v)) if k in HEADER_INT_FIELDS else repr(float(v)))
    n = g.n1 * g.n2
    cols = np.empty((n, VALUES_PER_CELL), dtype=np.float64)
    cols[:, 0] = ex["x1"].reshape(n)
    cols[:, 1] = ex["x2"].reshape(n)
    cols[:, 2] = ex["r"].reshape(n)
    cols[:, 3] = ex["th"].reshape(n)
    cols[:, 4:12] = dump.prims.reshape(8, n).T
    cols[:, 12] = 0.0
    cols[:, 13:17] = ex["ucon"].reshape(n, 4)
    cols[:, 17:21] = ex["ucov"].reshape(n, 4)
    cols[:, 21:25] = ex["bcon"].reshape(n, 4)
    cols[:, 25:29] = ex["bcov"].reshape(n, 4)
    cols[:, 29:33] = 0.0
    cols[:, 33] = ex["gdet"].reshape(n)
    with open(path, "w") as f:
        f.write(" ".join(parts) + "\n")
        np.savetxt(f, cols, fmt="%.17g")


def read_dump(path: str | os.PathLike, n1: int | None = None, n2: int | None = None) -> Dump:
    """Read a HARM ASCII dump into a Dump (prims [8][n1][n2] float64)."""
    with open(path, "r") as f:
        head = f.readline().split()
        if len(head) < len(HEADER_FIELDS):
            raise DumpFormatError(f"{path}: header has {len(head)} fields, expected {len(HEADER_FIELDS)}")
        hdr = {}
        for k, tok in zip(HEADER_FIELDS, head):
            hdr[k] = int(tok) if k in HEADER_INT_FIELDS else float(tok)
        dn1, dn2 = hdr["n1"], hdr["n2"]
        if n1 is not None and (dn1 != n1 or dn2 != n2):
            raise DumpFormatError(f"{path}: grid is {dn1}x{dn2}, expected {n1}x{n2}")
        if dn1 < 2 or dn2 < 2:
            raise DumpFormatError(f"{path}: grid {dn1}x{dn2} is too small for bilinear sampling")
        data = _parse_body(f)
    n = dn1 * dn2
    if data.size != n * VALUES_PER_CELL:
        raise DumpFormatError(f"{path}: {data.size} values for {n} cells "
                              f"(expected {n * VALUES_PER_CELL}); truncated or malformed dump")
    cols = data.reshape(n, VALUES_PER_CELL)
    prims = np.ascontiguousarray(cols[:, 4:12].T.reshape(8, dn1, dn2))
    if not np.all(np.isfinite(prims)):
        raise DumpFormatError(f"{path}: non-finite primitive values")
    geom = GridGeom(n1=dn1, n2=dn2, startx1=hdr["startx1"], startx2=hdr["startx2"],
                    dx1=hdr["dx1"], dx2=hdr["dx2"], a=hdr["a"], hslope=hdr["hslope"],
                    R0=hdr["R0"], Rin=hdr["Rin"], Rout=hdr["Rout"], gam=hdr["gam"])
    extras = dict(x1=cols[:, 0].reshape(dn1, dn2), x2=cols[:, 1].reshape(dn1, dn2),
                  r=cols[:, 2].reshape(dn1, dn2), th=cols[:, 3].reshape(dn1, dn2),
                  ucon=cols[:, 13:17].reshape(dn1, dn2, 4), ucov=cols[:, 17:21].reshape(dn1, dn2, 4),
                  bcon=cols[:, 21:25].reshape(dn1, dn2, 4), bcov=cols[:, 25:29].reshape(dn1, dn2, 4),
                  gdet=cols[:, 33].reshape(dn1, dn2))
    return Dump(geom=geom, prims=prims, extras=extras)


def _parse_body(f) -> np.ndarray:
    text = f.read()
    try:
        return np.array(text.split(), dtype=np.float64)
    except ValueError as e:
        raise DumpFormatError(f"malformed number in dump body: {e}") from None


@dataclasses.dataclass
class ModelIn:
    """The eleven model.in entries, in read_model's order (core.c:22-34)."""
    MBH: float = 8.9505e39
    M_UNIT: float = 1e19
    ABSORPTION: int = 1
    IMG_WIDTH: int = 100
    IMG_HEIGHT: int = 100
    CAM_SIZE_X: float = 40.0
    CAM_SIZE_Y: float = 40.0
    FREQS_PER_DEC: int = 1
    FREQ_MIN: float = 230e9
    FREQ_MAX: float = 230e9
    STEPSIZE: float = 0.05

    _UNITS = {"MBH": "(g)", "M_UNIT": "(g)", "ABSORPTION": "(-)", "IMG_WIDTH": "(pixels)",
              "IMG_HEIGHT": "(pixels)", "CAM_SIZE_X": "(Rg)", "CAM_SIZE_Y": "(Rg)",
              "FREQS_PER_DEC": "(-)", "FREQ_MIN": "(Hz)", "FREQ_MAX": "(Hz)", "STEPSIZE": "(-)"}
    _INTS = ("ABSORPTION", "IMG_WIDTH", "IMG_HEIGHT", "FREQS_PER_DEC")

    def write(self, path: str | os.PathLike) -> None:
        with open(path, "w") as f:
            for fld in dataclasses.fields(self):
                v = getattr(self, fld.name)
                s = str(int(v)) if fld.name in self._INTS else repr(float(v))
                f.write(f"{fld.name}\t{self._UNITS[fld.name]}\t{s}\n")

    @classmethod
    def read(cls, path: str | os.PathLike) -> "ModelIn":
        toks = open(path).read().split()
        names = [f.name for f in dataclasses.fields(cls)]
        if len(toks) < 3 * len(names):
            raise ValueError(f"{path}: model.in needs {len(names)} 'NAME (unit) value' lines")
        kw = {}
        for i, n in enumerate(names):
            v = toks[3 * i + 2]
            kw[n] = int(v) if n in cls._INTS else float(v)
        return cls(**kw)
