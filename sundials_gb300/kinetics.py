"""Seeded generator for the uneven stiff mass-action kinetics batch.

Each system i has n_i species, n_i ~ U{8..64}, and 2 n_i reactions.  A
reaction is unimolecular A -> B or bimolecular A + B -> C with probability
1/2 each; the species of one reaction are distinct and drawn uniformly; the
rate constant is log-uniform over [1e-2, 1e6]; the initial concentrations are
uniform[0, 1] normalised to sum 1.

Every draw comes from a counter-based SplitMix64 hash of (seed, stream,
counter), so any subset of systems can be regenerated independently and the
arrays are identical on every machine.

Right-hand side (the order of every floating-point sum is part of the
definition, so CPU and GPU evaluate the same bits):
  rate_r = k_r * y_A            (A -> B)
  rate_r = (k_r * y_A) * y_B    (A + B -> C)
  f_s    = sum over reactions r in index order of the signed rates that touch s
Jacobian: J[s][j] = sum over reactions r in index order of d(signed rate)/dy_j.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def _uniform(seed: int, stream: int, counter: np.ndarray) -> np.ndarray:
    """Uniform doubles in [0, 1) from (seed, stream, counter)."""
    with np.errstate(over="ignore"):
        key = _splitmix64(np.uint64(seed) * np.uint64(0x632BE59BD9B4E019)
                          + np.uint64(stream) * np.uint64(0x9E3779B97F4A7C15))
        z = _splitmix64(key ^ counter.astype(np.uint64))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class KineticsBatch:
    n: np.ndarray        # int32 [nsys]            species per system
    y_off: np.ndarray    # int64 [nsys+1]          offsets into y0
    r_off: np.ndarray    # int64 [nsys+1]          offsets into reactions
    rtype: np.ndarray    # int32 [R]               0: A->B, 1: A+B->C
    ra: np.ndarray       # int32 [R]               reactant A (local index)
    rb: np.ndarray       # int32 [R]               product B (uni) / reactant B (bi)
    rc: np.ndarray       # int32 [R]               product C (bi) or -1
    rk: np.ndarray       # float64 [R]             rate constant
    y0: np.ndarray       # float64 [sum n]         initial state

    @property
    def nsys(self) -> int:
        return int(self.n.size)

    def subset(self, idx) -> "KineticsBatch":
        idx = np.asarray(idx, dtype=np.int64)
        n = self.n[idx]
        y_off = np.zeros(idx.size + 1, np.int64)
        y_off[1:] = np.cumsum(n)
        r_off = np.zeros(idx.size + 1, np.int64)
        r_off[1:] = np.cumsum(2 * n.astype(np.int64))
        ysel = np.concatenate([np.arange(self.y_off[i], self.y_off[i + 1]) for i in idx])
        rsel = np.concatenate([np.arange(self.r_off[i], self.r_off[i + 1]) for i in idx])
        return KineticsBatch(n, y_off, r_off, self.rtype[rsel], self.ra[rsel], self.rb[rsel],
                             self.rc[rsel], self.rk[rsel], self.y0[ysel])


def generate(nsys: int = 65536, seed: int = 1, nmin: int = 8, nmax: int = 64,
             first: int = 0) -> KineticsBatch:
    """Systems first .. first+nsys-1 of the batch with this seed."""
    sys_ids = np.arange(first, first + nsys, dtype=np.uint64)
    n = (nmin + np.floor(_uniform(seed, 1, sys_ids) * (nmax - nmin + 1))).astype(np.int32)
    n = np.minimum(n, nmax)
    y_off = np.zeros(nsys + 1, np.int64)
    y_off[1:] = np.cumsum(n)
    nr = 2 * n.astype(np.int64)
    r_off = np.zeros(nsys + 1, np.int64)
    r_off[1:] = np.cumsum(nr)
    R = int(r_off[-1])
    # reaction counter = system id * 256 + local reaction index (2n <= 128)
    sys_of_r = np.repeat(np.arange(nsys), nr)
    local_r = np.arange(R, dtype=np.int64) - r_off[:-1][sys_of_r]
    ctr = (sys_ids[sys_of_r] << np.uint64(8)) + local_r.astype(np.uint64)
    nn = n[sys_of_r].astype(np.int64)
    rtype = (_uniform(seed, 2, ctr) >= 0.5).astype(np.int32)
    a = np.floor(_uniform(seed, 3, ctr) * nn).astype(np.int64)
    b = np.floor(_uniform(seed, 4, ctr) * (nn - 1)).astype(np.int64)
    b = b + (b >= a)
    c = np.floor(_uniform(seed, 5, ctr) * (nn - 2)).astype(np.int64)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    c = c + (c >= lo)
    c = c + (c >= hi)
    c = np.where(rtype == 1, c, -1)
    k = 10.0 ** (-2.0 + 8.0 * _uniform(seed, 6, ctr))
    # initial state: uniform[0,1) per species, normalised per system
    Y = int(y_off[-1])
    sys_of_y = np.repeat(np.arange(nsys), n)
    local_y = np.arange(Y, dtype=np.int64) - y_off[:-1][sys_of_y]
    yctr = (sys_ids[sys_of_y] << np.uint64(8)) + local_y.astype(np.uint64)
    y0 = _uniform(seed, 7, yctr)
    sums = np.zeros(nsys)
    for i in range(nsys):  # sequential sum per system (fixed order)
        s = 0.0
        for v in y0[y_off[i]:y_off[i + 1]]:
            s += v
        sums[i] = s
    y0 = y0 / sums[sys_of_y]
    return KineticsBatch(n, y_off, r_off, rtype, a.astype(np.int32), b.astype(np.int32),
                         c.astype(np.int32), k, y0)


def rhs(batch: KineticsBatch, i: int, y: np.ndarray) -> np.ndarray:
    """f(y) of system i in the defined summation order (a slow reference)."""
    n = int(batch.n[i])
    f = np.zeros(n)
    r0, r1 = batch.r_off[i], batch.r_off[i + 1]
    for r in range(r0, r1):
        A, B, Cc, k = batch.ra[r], batch.rb[r], batch.rc[r], batch.rk[r]
        if batch.rtype[r] == 0:
            rate = k * y[A]
            f[A] = f[A] - rate
            f[B] = f[B] + rate
        else:
            rate = (k * y[A]) * y[B]
            f[A] = f[A] - rate
            f[B] = f[B] - rate
            f[Cc] = f[Cc] + rate
    return f


# ------------------------------------------------------------- file format
STATS_FIELDS = ["nst", "nfe", "nsetups", "nje", "nni", "ncfn", "netf", "nnf", "flag", "qu"]
STATS_DTYPE = np.dtype([(f, "<i8") for f in STATS_FIELDS] + [("tn", "<f8"), ("hu", "<f8")])
# SUNBatchBDFStats (include/sunbatchbdf_gb300.h): the drivers' fields plus the
# three CVodePrintAllStats needs
BATCH_STATS_DTYPE = np.dtype(STATS_DTYPE.descr + [("h0u", "<f8"), ("next_h", "<f8"),
                                                  ("next_q", "<i8")])


def write_bin(batch: KineticsBatch, path) -> None:
    """Problem file read by the C drivers (layout in oracle/kinetics_model.h)."""
    with open(path, "wb") as f:
        np.array([batch.nsys, batch.y0.size, batch.rk.size], "<i8").tofile(f)
        batch.n.astype("<i4").tofile(f)
        batch.y_off.astype("<i8").tofile(f)
        batch.r_off.astype("<i8").tofile(f)
        for a in (batch.rtype, batch.ra, batch.rb, batch.rc):
            a.astype("<i4").tofile(f)
        batch.rk.astype("<f8").tofile(f)
        batch.y0.astype("<f8").tofile(f)


def read_results(path, batch: KineticsBatch):
    """(stats structured array, y list) from a driver's output file."""
    raw = open(path, "rb").read()
    stats = np.zeros(batch.nsys, STATS_DTYPE)
    ys = []
    off = 0
    for i in range(batch.nsys):
        stats[i] = np.frombuffer(raw, STATS_DTYPE, 1, off)[0]
        off += STATS_DTYPE.itemsize
        n = int(batch.n[i])
        ys.append(np.frombuffer(raw, "<f8", n, off).copy())
        off += 8 * n
    return stats, ys
