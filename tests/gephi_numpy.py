"""A second, independent CPU restatement of the ForceAtlas2 iteration, in
numpy: the plain transcription of Gephi's algorithm that the reference's own
tests check their C code against (reference
tests/testthat/helper-reference.R:3-100). Exact O(n^2) repulsion, gravity,
an edge loop, Gephi's adaptive speed and the displacement, in that order.

Test infrastructure only: it checks the C oracle (oracle/fa2_oracle.c) with
code written independently of it, as the reference's tests check
src/forceatlas2.c with their R transcription.
"""
from __future__ import annotations

import numpy as np


def gephi_layout(n, frm, to, pos, iterations, scaling, gravity=1.0,
                 strong=False, linlog=False, outbound=False, adjust=False,
                 size=1.0, w=None, jt_user=1.0, fixed=None):
    """Positions after `iterations` steps (helper-reference.R:3-100), for an
    edge list with 0-based ends; `pos` is n x 2."""
    frm = np.asarray(frm, np.int64)
    to = np.asarray(to, np.int64)
    m = len(frm)
    w = np.ones(m) if w is None else np.asarray(w, np.float64)
    fixed = np.zeros(n, bool) if fixed is None else np.asarray(fixed, bool)
    size = np.broadcast_to(np.asarray(size, np.float64), (n,)).copy()
    # every edge end counts, a self-loop twice (helper-reference.R:15)
    mass = 1.0 + np.bincount(np.concatenate([frm, to]), minlength=n).astype(np.float64)
    x = np.array(pos[:, 0], np.float64)
    y = np.array(pos[:, 1], np.float64)
    dx = np.zeros(n)
    dy = np.zeros(n)
    speed, eff = 1.0, 1.0
    mm = np.outer(mass, mass)
    ss = size[:, None] + size[None, :]
    off_diag = ~np.eye(n, dtype=bool)

    for _ in range(iterations):
        odx, ody = dx, dy

        # repulsion: f = s m_i m_j / d^2 (adjust: d minus both radii, 100 s
        # m_i m_j on overlap), nothing at d = 0 or on the diagonal
        xd = x[:, None] - x[None, :]
        yd = y[:, None] - y[None, :]
        d = np.sqrt(xd * xd + yd * yd)
        with np.errstate(divide="ignore", invalid="ignore"):
            if adjust:
                d = d - ss
                f = np.where(d > 0, scaling * mm / (d * d),
                             np.where(d < 0, 100.0 * scaling * mm, 0.0))
            else:
                f = np.where(d > 0, scaling * mm / (d * d), 0.0)
        f = np.where(off_diag, f, 0.0)
        dx = (xd * f).sum(axis=1)
        dy = (yd * f).sum(axis=1)

        # gravity
        d0 = np.sqrt(x * x + y * y)
        if strong:
            g = gravity * mass
        else:
            with np.errstate(divide="ignore", invalid="ignore"):
                g = np.where(d0 > 0, gravity * mass / d0, 0.0)
        dx = dx - x * g
        dy = dy - y * g

        # attraction, edge by edge
        coef = mass.mean() if outbound else 1.0
        for e in range(m):
            i, j = frm[e], to[e]
            ex = x[i] - x[j]
            ey = y[i] - y[j]
            fe = -coef * w[e]
            if adjust or linlog:
                de = np.sqrt(ex * ex + ey * ey)
                if adjust:
                    de = de - size[i] - size[j]
                if de <= 0:
                    continue
                if linlog:
                    fe = fe * np.log1p(de) / de
            if outbound:
                fe = fe / mass[i]
            dx[i] += ex * fe
            dy[i] += ey * fe
            dx[j] -= ex * fe
            dy[j] -= ey * fe

        # Gephi's adaptive speed
        swing_i = mass * np.sqrt((odx - dx) ** 2 + (ody - dy) ** 2)
        swing = swing_i[~fixed].sum()
        tract = (0.5 * mass * np.sqrt((odx + dx) ** 2 + (ody + dy) ** 2))[~fixed].sum()
        est = 0.05 * np.sqrt(n)
        jt = jt_user * max(np.sqrt(est), min(10.0, est * tract / (n * n)))
        if swing / tract > 2:
            if eff > 0.05:
                eff *= 0.5
            jt = max(jt, jt_user)
        target = jt * eff * tract / swing
        if swing > jt * tract:
            if eff > 0.05:
                eff *= 0.7
        elif speed < 1000:
            eff *= 1.3
        speed = speed + min(target - speed, 0.5 * speed)

        # displacement
        if adjust:
            fac = 0.1 * speed / (1.0 + np.sqrt(speed * swing_i))
            df = np.sqrt(dx * dx + dy * dy)
            with np.errstate(divide="ignore", invalid="ignore"):
                fac = np.where(df == 0, 0.0, np.minimum(fac * df, 10.0) / df)
        else:
            fac = speed / (1.0 + np.sqrt(speed * swing_i))
        fac = np.where(fixed, 0.0, fac)
        x = x + dx * fac
        y = y + dy * fac
    return np.column_stack([x, y])


def mean_rel(current, target):
    """The relative difference testthat's expect_equal(tolerance = ...)
    compares: sum |target - current| / sum |target|."""
    current = np.asarray(current, np.float64)
    target = np.asarray(target, np.float64)
    return np.abs(target - current).sum() / np.abs(target).sum()
