"""saveat / save_start / save_end resolution with the reference's rules.

* A number saveat d means the range (t0 + tdir|d|):(tdir|d|):tf (lib/OrdinaryDiffEqCore/src/solve.jl:1103-1124),
  evaluated like Julia's Float64 range: when start, step and stop have exact
  small rational forms the elements are the correctly rounded rationals (so
  0.1:0.1:1.0 gives 0.3, not 0.1 + 0.2).
* A vector saveat keeps the entries in (t0, tf] ([tf, t0) backward; the device skips
  the rest).  The points are passed ascending whatever the direction.
* Defaults (solve.jl:141-143, 596-599): save_start = isempty(saveat) || saveat is a
  number || t0 in saveat; save_end = isempty(saveat) || saveat is a number ||
  tf in saveat; save_everystep makes both true.  save_everystep with saveat
  keeps both sets (_savevalues!: the saveat points up to t, then the step
  unless a saveat point landed on it).
"""
from dataclasses import dataclass
from fractions import Fraction

import numpy as np

_MAXINTFLOAT32 = 16777216  # maxintfloat(Float32), the bound Base.rat uses for Float64


def julia_rat(x):
    """Base.rat(x::Float64): continued-fraction rational with |num|,|den| <= 2^24."""
    y = x
    a, d = 1, 1
    b, c = 0, 0
    m = _MAXINTFLOAT32
    while abs(y) <= m:
        f = int(y)  # trunc
        y -= f
        a, c = f * a + c, a
        b, d = f * b + d, b
        if max(abs(a), abs(b)) > m:
            return c, d
        if b != 0 and float(a) / float(b) == x:
            break
        if y == 0:
            break
        y = 1.0 / y
    return a, b


def _between(a, x, b):
    # Base.isbetween: x between a and b in either order
    return a <= x <= b or b <= x <= a


def julia_float_range(start, step, stop):
    """Elements of Julia's start:step:stop for Float64 (Base (:) on IEEE floats)."""
    if step == 0:
        raise ValueError("range step cannot be zero")
    sn, sd = julia_rat(step)
    if sd != 0 and sn / sd == step:
        an, ad = julia_rat(start)
        zn, zd = julia_rat(stop)
        if ad != 0 and zd != 0 and an / ad == start and zn / zd == stop:
            den = ad * sd // np.gcd(ad, sd)
            start_n = round(start * den)
            step_n = round(step * den)
            if step_n != 0:
                length = max(0, (den * zn - zd * start_n + step_n * zd) // (step_n * zd))
                last = Fraction(start_n + (length - 1) * step_n, den)
                nxt = Fraction(start_n + length * step_n, den)
                if length > 0 and _between(Fraction(start), last, Fraction(stop) + Fraction(step) / 2) \
                        and not _between(Fraction(start), nxt, Fraction(stop)):
                    return np.array([float(Fraction(start_n + k * step_n, den)) for k in range(length)])
    lf = (stop - start) / step
    if lf < 0:
        n = 0
    elif lf == 0:
        n = 1
    else:
        n = int(round(lf)) + 1
        stop2 = start + (n - 1) * step
        n -= int(start < stop < stop2) + int(start > stop > stop2)
    return np.array([start + k * step for k in range(n)])


@dataclass
class SaveSpec:
    values: np.ndarray
    nsave: int
    per_traj: bool
    scalar: bool
    save_start: bool
    save_end: bool
    save_end_user: int
    everystep: bool = False      # save every accepted step (beside the saveat points, if any)
    max_step_saves: int = 0      # step saves kept per trajectory when everystep

    @property
    def cap(self):
        """Output slots per trajectory: t_out is (cap, N), u_out (cap, n, N)."""
        return self.nsave + (self.max_step_saves if self.everystep else 0) + 2


def resolve_saveat(saveat, tspans, save_start=None, save_end=None, save_everystep=False, max_step_saves=1024):
    """tspans: (2, N).  Returns the SaveSpec passed to the C ABI (a SaveSpec is
    returned unchanged).  save_everystep keeps every accepted step, up to
    max_step_saves per trajectory, beside the saveat points if any."""
    if isinstance(saveat, SaveSpec):
        return saveat
    no_saveat = saveat is None or (not np.isscalar(saveat) and np.size(saveat) == 0)
    if save_everystep and not no_saveat:
        if max_step_saves <= 0:
            raise ValueError("save_everystep needs max_step_saves > 0")
        # the saveat points as without it, with save_start and save_end true by default
        sv = resolve_saveat(saveat, tspans, True if save_start is None else save_start,
                            True if save_end is None else save_end)
        sv.save_end_user = -1 if save_end is None else int(bool(save_end))
        sv.everystep = True
        sv.max_step_saves = int(max_step_saves)
        return sv
    if save_everystep:
        if max_step_saves <= 0:
            raise ValueError("save_everystep needs max_step_saves > 0")
        return SaveSpec(np.zeros(0), 0, False, False, True if save_start is None else bool(save_start),
                        True if save_end is None else bool(save_end), -1 if save_end is None else int(bool(save_end)),
                        True, int(max_step_saves))
    tspans = np.asarray(tspans, dtype=np.float64)
    t0s, tfs = tspans[0], tspans[1]
    same_span = bool(np.all(t0s == t0s[0]) and np.all(tfs == tfs[0])) if tspans.shape[1] else True
    seu = -1 if save_end is None else int(bool(save_end))
    if tspans.shape[1] == 0:  # empty ensemble: nothing to resolve
        return SaveSpec(np.zeros(0), 0, False, np.isscalar(saveat), True if save_start is None else bool(save_start),
                        True if save_end is None else bool(save_end), seu)
    if saveat is None or (not np.isscalar(saveat) and np.size(saveat) == 0):
        return SaveSpec(np.zeros(0), 0, False, False, True if save_start is None else bool(save_start),
                        True if save_end is None else bool(save_end), seu)
    if np.isscalar(saveat):
        # (t0 + tdir|d|):(tdir|d|):tf, stored ascending (the device reads a
        # backward trajectory's points from the end)
        d = abs(float(saveat))
        sd = lambda a, b: -d if b < a else d
        if same_span:
            vals = np.sort(julia_float_range(t0s[0] + sd(t0s[0], tfs[0]), sd(t0s[0], tfs[0]), tfs[0]))
            per = False
        else:
            rows = [np.sort(julia_float_range(a + sd(a, b), sd(a, b), b)) for a, b in zip(t0s, tfs)]
            m = max(len(r) for r in rows)
            vals = np.full((m, len(rows)), np.inf)
            for j, r in enumerate(rows):
                vals[:len(r), j] = r
            per = True
        return SaveSpec(np.ascontiguousarray(vals), vals.shape[0], per, True,
                        True if save_start is None else bool(save_start),
                        True if save_end is None else bool(save_end), seu)
    arr = np.asarray(saveat, dtype=np.float64)
    if arr.ndim == 1:
        vals = np.sort(arr)
        ss = [float(t0s[0]) in set(vals.tolist())] if same_span else [a in set(vals.tolist()) for a in t0s]
        se = [float(tfs[0]) in set(vals.tolist())] if same_span else [b in set(vals.tolist()) for b in tfs]
        per = False
    else:
        vals = np.sort(arr, axis=0)
        ss = [t0s[j] in set(vals[:, j].tolist()) for j in range(vals.shape[1])]
        se = [tfs[j] in set(vals[:, j].tolist()) for j in range(vals.shape[1])]
        per = True
    if save_start is None:
        if len(set(ss)) > 1:
            raise ValueError("save_start differs between trajectories; pass save_start explicitly")
        save_start = ss[0] if ss else False
    if save_end is None:
        if len(set(se)) > 1:
            raise ValueError("save_end differs between trajectories; pass save_end explicitly")
        save_end = se[0] if se else False
    return SaveSpec(np.ascontiguousarray(vals), vals.shape[0], per, False, bool(save_start), bool(save_end), seu)
