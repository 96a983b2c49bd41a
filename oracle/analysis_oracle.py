"""ORACLE -- test infrastructure only.  FP64 restatement of the reference's
offline analysis, which the library's observables replace:

  Stat<T>::Compute                analyze/statistics.h:35-54
  Stat<T>::Find_Correlation_Length analyze/statistics.h:68-82
  Compute_Order_Parameters        analyze/analyze.h:121-146
  Pair_Distribution               analyze/analyze.h:365-424 (one frame, counts)

The arithmetic follows the reference's order of operations (sequential
sums, each autocorrelation term divided by (T - tau) before it is added), so
that on the same series the library's host code agrees bit for bit.
Pure-Python loops: for series and particle counts that finish in seconds."""
import math

import numpy as np


def stat_compute(data):
    """mean, mean_square, variance, std, min, max, corr_len, error of a series."""
    data = [float(v) for v in data]
    T = len(data)
    mn = mx = data[0]
    for v in data:
        mx = v if mx < v else mx
        mn = v if mn > v else mn
    s = 0.0
    for v in data:
        s += v
    sq = 0.0
    for v in data:
        sq += v * v
    mean = s / T
    mean_square = sq / T
    variance = mean_square - mean * mean
    corr_len = 0.0
    for tau in range(T // 2):
        c = 0.0
        for i in range(T - tau):
            c += (data[i] - mean) * (data[i + tau] - mean) / (T - tau)
        c = c / variance if variance != 0 else math.nan
        corr_len = float(tau)
        if c < 0.01:
            break
    error = math.sqrt(variance * corr_len / T)
    return dict(mean=mean, mean_square=mean_square, variance=variance, std=math.sqrt(variance), min=mn,
                max=mx, corr_len=corr_len, error=error)


def order_parameters(p, area):
    """Compute_Order_Parameters on per-frame polarizations p: <P>, its error,
    sigma2 = variance * area, and G as the reference writes it
    (1 - <P^4>/(3<P^2>)) next to the standard Binder cumulant."""
    st = stat_compute(p)
    s4 = 0.0
    for v in p:
        s4 += (v * v) * (v * v)
    p4 = s4 / len(p)
    st.update(sigma2=st["variance"] * area, p4_mean=p4,
              binder_reference=1 - p4 / (3 * st["mean_square"]),
              binder=1 - p4 / (3 * st["mean_square"] ** 2))
    return st


def frame_polarization(theta):
    """P of one frame from the headings (FP64 cos/sin, analyze.h:127-139)."""
    th = np.asarray(theta, np.float64)
    return math.hypot(np.cos(th).sum() / len(th), np.sin(th).sum() / len(th))


def pair_distribution(x, y, theta, lx, ly, gx, gy):
    """Counts of one frame of Pair_Distribution: ordered pairs (j, k), the
    plain difference r_k - r_j in the frame of j's heading."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    c = np.cos(np.asarray(theta, np.float64))
    s = np.sin(np.asarray(theta, np.float64))
    counts = np.zeros((gx, gy), np.int64)
    for j in range(len(x)):
        dx = x - x[j]
        dy = y - y[j]
        ty = c[j] * dx + s[j] * dy
        tx = s[j] * dx - c[j] * dy
        ok = (np.abs(tx) < lx) & (np.abs(ty) < ly)
        ok[j] = False
        bx = (gx * ((tx[ok] / lx) + 1) / 2).astype(np.int64)
        by = (gy * ((ty[ok] / ly) + 1) / 2).astype(np.int64)
        np.add.at(counts, (bx, by), 1)
    return counts


def radial_counts(x, y, L, r_max, nbins):
    """Ordered-pair minimum-image distance histogram in FP64."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    counts = np.zeros(nbins, np.int64)
    dr = r_max / nbins
    for i in range(len(x)):
        dx = x - x[i]
        dy = y - y[i]
        dx -= 2 * L * np.round(dx / (2 * L))
        dy -= 2 * L * np.round(dy / (2 * L))
        d = np.hypot(dx, dy)
        d[i] = np.inf
        b = np.minimum((d[d < r_max] / dr).astype(np.int64), nbins - 1)
        np.add.at(counts, b, 1)
    return counts


def ring_shape(x, y):
    """Box::Compute_All_Variables' shape quantities (parallel/beadbox.h:
    402-428) of one set of unwrapped points: cm, xx, yy, xy, lambda1,
    lambda2, Rg, Delta (FP64)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n = len(x)
    cx, cy = x.sum() / n, y.sum() / n
    xx = (x * x).sum() / n - cx * cx
    yy = (y * y).sum() / n - cy * cy
    xy = (x * y).sum() / n - cx * cy
    root = math.sqrt((xx - yy) ** 2 + 4 * xy * xy)
    l1 = 0.5 * (xx + yy) + 0.5 * root
    l2 = 0.5 * (xx + yy) - 0.5 * root
    return dict(cm_x=cx, cm_y=cy, xx=xx, yy=yy, xy=xy, lambda1=l1, lambda2=l2, Rg=math.sqrt(xx + yy),
                Delta=((l1 - l2) / (l1 + l2)) ** 2)


def ring_motion(mb_now, mb_old, sw_now, sw_old, th_now, th_old, elapsed):
    """Box::Compute_All_Variables' motion terms (parallel/beadbox.h:325-434)
    of one vesicle in FP64, from the unwrapped positions (x, y) of its
    membrane beads and swimmers now and at the marked frame, the swimmers'
    headings then and now, and the time between the frames: the centre-of-
    mass velocities, the angular momenta, the rotation rates and the mean
    swimmer spin (the heading change folded as the reference folds it)."""
    mx, my = (np.asarray(a, np.float64) for a in mb_now)
    ox, oy = (np.asarray(a, np.float64) for a in mb_old)
    sx, sy = (np.asarray(a, np.float64) for a in sw_now)
    px, py = (np.asarray(a, np.float64) for a in sw_old)
    Nm, Ns = len(mx), len(sx)
    mvx, mvy = (mx - ox) / elapsed, (my - oy) / elapsed
    svx, svy = (sx - px) / elapsed, (sy - py) / elapsed
    dth = np.asarray(th_now, np.float64) - np.asarray(th_old, np.float64)
    dth -= 2 * math.pi * np.floor(dth / (2 * math.pi))
    dth -= 2 * math.pi * np.floor(dth / math.pi)
    mcx, mcy = mx.sum() / Nm, my.sum() / Nm
    scx, scy = sx.sum() / Ns, sy.sum() / Ns
    mb_v = (mvx.sum() / Nm, mvy.sum() / Nm)
    sw_v = (svx.sum() / Ns, svy.sum() / Ns)
    mxx = (mx * mx).sum() / Nm - mcx * mcx
    myy = (my * my).sum() / Nm - mcy * mcy
    sxx = (sx * sx).sum() / Ns - scx * scx
    syy = (sy * sy).sum() / Ns - scy * scy
    mb_l = (mx * mvy - my * mvx).sum() / Nm - mcx * mb_v[1] + mcy * mb_v[0]
    sw_l = ((sx * svy - sy * svx).sum() / Ns - scx * mb_v[1] + scy * mb_v[0] - mcx * sw_v[1] + mcy * sw_v[0]
            + mcx * mb_v[1] - mcy * mb_v[0])
    return dict(mb_v_cm_x=mb_v[0], mb_v_cm_y=mb_v[1], mb_l=mb_l, mb_omega=mb_l / (mxx + myy),
                sw_v_cm_x=sw_v[0], sw_v_cm_y=sw_v[1], sw_l=sw_l,
                sw_omega=sw_l / (sxx + syy + (mcx - scx) ** 2 + (mcy - scy) ** 2),
                sw_spin=(dth / elapsed).sum() / Ns)
