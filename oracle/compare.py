"""TEST INFRASTRUCTURE ONLY: parity checks of GPU results against the oracle.

Parity definition for this path:
* integer FFT-CC displacements equal the oracle's, except at peaks that tie:
  an exact tie is two shifts with equal exact (integer) correlation; a
  rounding tie is a pair whose exact correlation values differ by less than
  the FP32 DFT rounding bound (`tie_rtol` of the correlation range), where the
  oracle's own FP32 arithmetic cannot decide the order.  Both are counted and
  reported; any other mismatch is a failure;
* sub-pixel u, v within 1e-3 px and displacement gradients within 1e-5 of
  the oracle's FP32 restatement of the reference CPU path, on POIs both flag
  Success with the same iteration count; flags equal.  A POI whose iteration
  count differs is a convergence-threshold tie: counted, u, v still within
  1e-3 px, gradients within the last-step bound delta_p / r, at most 1% of
  the POIs.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import oracle as O

UV_TOL = 1e-3
GRAD_TOL = 1e-5
# ZNCC: the FP32 oracle's own rounding reaches ~1e-5 for 62x62 windows (sums
# of squares near 1e7 in float), so the bound is 3e-5
ZNCC_TOL = 3e-5


@dataclasses.dataclass
class FftccReport:
    n: int
    mismatches: int
    exact_ties: int
    rounding_ties: int
    unexplained: int
    max_zncc_err: float

    def ok(self):
        return self.unexplained == 0 and self.max_zncc_err <= ZNCC_TOL


def fftcc_parity(ref, tar, poi, r, u, v, z, u_or, v_or, z_or, st_or, tie_rtol=1e-5, ry=None) -> FftccReport:
    """r: window half width (and height unless ry is given)."""
    ok = st_or == 0
    mis = ok & ((u != u_or) | (v != v_or))
    exact = rounding = unexplained = 0
    ry = r if ry is None else ry
    for i in np.nonzero(mis)[0]:
        c = O.exact_surface(ref, tar, poi[i, 0], poi[i, 1], r, ry=ry)
        a = c[int(v[i]) % (2 * ry), int(u[i]) % (2 * r)]
        b = c[int(v_or[i]) % (2 * ry), int(u_or[i]) % (2 * r)]
        span = float(c.max() - c.min()) or 1.0
        if a == b:
            exact += 1
        elif abs(float(a) - float(b)) <= tie_rtol * span:
            rounding += 1
        else:
            unexplained += 1
    same = ok & ~mis
    zerr = float(np.abs(z[same] - z_or[same]).max()) if same.any() else 0.0
    return FftccReport(int(ok.sum()), int(mis.sum()), exact, rounding, unexplained, zerr)


@dataclasses.dataclass
class IcgnReport:
    n: int
    compared: int
    flag_mismatch: int
    iter_mismatch: int      # convergence-threshold ties (iteration counts differ)
    max_du: float
    max_dv: float
    max_dgrad: float        # over POIs with equal iteration counts
    over_uv: int
    over_grad: int          # equal-count POIs beyond GRAD_TOL
    over_tie_grad: int      # tie POIs beyond the last-step bound DELTA_P / r
    tie_limit: int

    def ok(self, grad_tol=GRAD_TOL):
        return (self.flag_mismatch == 0 and self.over_uv == 0 and self.over_grad == 0 and self.over_tie_grad == 0
                and self.iter_mismatch <= self.tie_limit)


def icgn_parity(p6, iters, flags, p6_or, iters_or, flags_or, mask=None, r=None, delta_p=1e-3) -> IcgnReport:
    """IC-GN parity.  A POI whose iteration count differs from the oracle's
    stopped on the other side of the ||dP|| >= delta_p test because of FP32
    rounding (a convergence-threshold tie, the analogue of an FFT-CC peak
    tie): it is counted, its u, v must still be within UV_TOL and its
    gradients within the last step's bound delta_p / r, and such ties must
    be rare (at most 1% of the POIs, plus one)."""
    m = np.ones(len(flags), bool) if mask is None else mask.copy()
    fm = int((m & (flags != flags_or)).sum())
    both = m & (flags == 0) & (flags_or == 0)
    same_it = both & (iters == iters_or)
    tie = both & (iters != iters_or)
    d = np.abs(p6.astype(np.float64) - p6_or.astype(np.float64))
    dg = d[:, [1, 2, 4, 5]].max(axis=1)
    du = float(d[both, 0].max()) if both.any() else 0.0
    dv = float(d[both, 3].max()) if both.any() else 0.0
    dgs = float(dg[same_it].max()) if same_it.any() else 0.0
    over_uv = int(((d[:, 0] > UV_TOL) | (d[:, 3] > UV_TOL))[both].sum())
    over_g = int((dg > GRAD_TOL)[same_it].sum())
    rr = 1.0 if r is None else float(r)
    over_tie = int((dg > delta_p / rr)[tie].sum())
    return IcgnReport(int(m.sum()), int(both.sum()), fm, int(tie.sum()), du, dv, dgs, over_uv, over_g, over_tie,
                      int(0.01 * int(both.sum())) + 1)


def truth_error(pair, poi, p6, flags):
    """Error of the sub-pixel result against the imposed synthetic field."""
    X, Y = poi[:, 1].astype(np.float64), poi[:, 0].astype(np.float64)
    uu, vv = pair.field(X, Y)
    ok = flags == 0
    eu = np.abs(p6[ok, 0] - uu[ok])
    ev = np.abs(p6[ok, 3] - vv[ok])
    return dict(mean_abs_u=float(eu.mean()), mean_abs_v=float(ev.mean()), max_abs_u=float(eu.max()),
                max_abs_v=float(ev.max()), rms=float(np.sqrt(np.mean(eu ** 2 + ev ** 2))))
