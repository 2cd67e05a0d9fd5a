"""Inputs that sit inside the safety margins of the kernels' single-precision
decision filters (test infrastructure).

The CUDA kernels decide TENO stencil selections and shock sensors first in
single precision and hand a decision to the exact double-precision
expression of the reference only when a quotient lies within a margin of its
cut-off (1e-4 relative for stencil selections, 1e-3 for the sensor's
interval filter and for the exponent arguments of the TENO-LAD and sensor
cut-offs).  Random fields almost never land there, so these helpers build
pencils that do: a smooth (triangle-wave) baseline plus a jump whose height
is tuned by bisection so that a chosen quotient equals its cut-off, then
perturbed by a spread of tiny relative amounts so that both sides of the
cut-off and both decision paths occur.

The quotients are evaluated with a numpy restatement of the reference's
formulas (TENOsensor::TENOA and TENOLAD_Op smoothness measures and weights,
src/prometeo_metric.inl:323-347, :351-403, :442-467, :1022-1038): it only
places inputs; the decisions themselves are compared between the GPU and the
CPU oracle.
"""
import math

import numpy as np

P10 = np.array([1e0, 1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12, 1e-13],
               dtype=np.float32).astype(np.float64)


def smoothness(w):
    """Smoothness measures s1..s4 and tau6 of windows w[..., 6] = (ym2 .. yp3)
    (src/prometeo_metric.inl:442-449)."""
    ym2, ym1, y, yp1, yp2, yp3 = (w[..., k] for k in range(6))
    C13, C23, C14, C24, C34 = 13.0 / 12.0, 3.0 / 12.0, 1.0 / 36.0, 13.0 / 12.0, 781.0 / 720.0
    s1 = C13 * (ym1 - 2 * y + yp1) ** 2 + C23 * (ym1 - yp1) ** 2
    s2 = C13 * (y - 2 * yp1 + yp2) ** 2 + C23 * (3 * y - 4 * yp1 + yp2) ** 2
    s3 = C13 * (ym2 - 2 * ym1 + y) ** 2 + C23 * (3 * y - 4 * ym1 + ym2) ** 2
    s4 = (C14 * (-11 * y + 18 * yp1 - 9 * yp2 + 2 * yp3) ** 2 + C24 * (2 * y - 5 * yp1 + 4 * yp2 - yp3) ** 2
          + C34 * (-y + 3 * yp1 - 3 * yp2 + yp3) ** 2)
    tau6 = np.abs(s4 - (s3 + s2 + 4 * s1) / 6)
    return np.stack([s1, s2, s3, s4], axis=-1), tau6


def quotients(w, eps):
    """q_k = a_k / sum_j a_j with a_k = (1 + tau6/(s_k + eps))^6, and chi_k."""
    s, tau6 = smoothness(w)
    chi = tau6[..., None] / (s + eps)
    a = (1.0 + chi) ** 6
    return a / a.sum(axis=-1, keepdims=True), chi


def sensor_cut_argument(phi):
    """Argument of the sensor's cut-off exponent, floor() of it is the power
    (src/prometeo_metric.inl:395-397): 12.5 - 11.5 (1 - (1-phi)^12 (1+12 phi))."""
    decay = (1.0 - phi) ** 12 * (1.0 + 12.0 * phi)
    return 12.5 - 11.5 * (1.0 - decay)


def sensor_cut(phi):
    z = sensor_cut_argument(phi)
    return P10[np.clip(np.floor(z).astype(int), 0, 13)]


def lad_argument(chi_max):
    """Argument of the TENO-LAD cut-off exponent, 3 + 9.5 / (1 + 0.1 chi_max)."""
    return 3.0 + 9.5 / (1.0 + chi_max * 0.1)


def bisect(f, lo, hi, iters=200):
    """Root of an increasing-or-decreasing f on [lo, hi] (sign change)."""
    flo = f(lo)
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        fm = f(mid)
        if (fm > 0) == (flo > 0):
            lo, flo = mid, fm
        else:
            hi = mid
        if hi - lo <= 1e-17 * abs(hi):
            break
    return 0.5 * (lo + hi)


def pencil(nx, j0, t, base=1.0, slope=0.02, jump=0.2):
    """Triangle-wave baseline (its kinks at 0 and nx/2, away from the jump)
    plus a jump of height t*jump between cells j0-1 and j0."""
    j = np.arange(nx, dtype=np.float64)
    tri = base + slope * np.minimum(j, nx - j)
    return tri + t * jump * (j >= j0)


def window(p, c):
    """Window (c-2 .. c+3) of a periodic pencil p: the stencil of the face
    c+1/2 (right-going side) and of the sensor node c."""
    n = len(p)
    return np.array([p[(c + k) % n] for k in range(-2, 4)])


def crossing_t(nx, j0, target, quantity, t_lo=1e-6, t_hi=1e3):
    """t at which quantity(window of node j0-1 of pencil(nx, j0, t)) equals
    `target`, found by bisection in log t."""
    c = j0 - 1
    f = lambda lt: quantity(window(pencil(nx, j0, math.exp(lt)), c)) - target
    return math.exp(bisect(f, math.log(t_lo), math.log(t_hi)))


def spread(n, lo=1e-9, hi=3e-2):
    """n relative offsets, log-spaced in [lo, hi], alternating in sign."""
    mags = np.geomspace(lo, hi, (n + 1) // 2)
    out = np.empty(n)
    out[0::2] = mags[: len(out[0::2])]
    out[1::2] = -mags[: len(out[1::2])]
    return out


def sensor_field(nx, ny, nz, phi_cut, seed=0):
    """rho pencils along x and a per-pencil Ducros value for the shock sensor
    of direction X (single species: Conserved[0] = rho).

    The first half of the (y, z) pencils holds the sensor's minimum quotient
    at the node before the jump within a spread of its cut-off (Ducros
    `phi_cut` for all of them); the second half has a smooth rho and Ducros
    values whose cut-off argument lies within a spread of an integer, so the
    cut-off exponent is decided at its margin.  Returns rho[z, y, x],
    phi[z, y, x] and the predicted numbers of nodes that must take the
    exact path (sensor quotient, cut-off argument)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    npen = ny * nz
    half = npen // 2
    j0 = nx // 4
    cut = float(sensor_cut(phi_cut))
    qmin = lambda w: float(quotients(w, 1e-8)[0].min())
    t_star = crossing_t(nx, j0, cut, qmin)
    rho = np.empty((npen, nx))
    phi = np.empty((npen, nx))
    d = spread(half, 1e-10, 1e-2)
    for i in range(half):
        rho[i] = pencil(nx, j0, t_star * (1 + d[i]))
        phi[i] = phi_cut
    # Ducros values whose cut-off argument crosses integers 7 .. 11
    n2 = npen - half
    targets = np.arange(7, 12)
    d2 = spread(n2, 1e-9, 1e-3)
    for i in range(n2):
        m = targets[i % len(targets)]
        ph = bisect(lambda x: sensor_cut_argument(x) - m, 0.0, 1.0)
        rho[half + i] = pencil(nx, j0, 0.0) * (1 + 0.01 * rng.uniform(-1, 1))
        phi[half + i] = ph * (1 + d2[i])
    q_near = 0
    for i in range(half):
        for c in range(nx):
            q = quotients(window(rho[i], c), 1e-8)[0]
            if np.all(q > cut * (1 - 1e-3)) and np.any(np.abs(q / cut - 1) < 5e-5):
                q_near += 1
    z = sensor_cut_argument(phi[half:, 0])
    cut_near = int(np.sum(np.abs(z - np.round(z)) < 5e-4)) * nx
    return (rho.reshape(nz, ny, nx), phi.reshape(nz, ny, nx), q_near, cut_near)


def teno_lad_field(nx, ny, nz):
    """rho pencils along x whose TENO-LAD cut-off argument at face j0-1/2+1
    (right-going side) lies within a spread of the integers 5 .. 11."""
    npen = ny * nz
    j0 = nx // 4
    targets = np.arange(5, 12)
    chi_max = lambda w: float(quotients(w, 1e-16)[1].max())
    d = spread(npen, 1e-10, 1e-2)
    t_of = {int(m): crossing_t(nx, j0, 10.0 * ((9.5 / (m - 3.0)) - 1.0), chi_max) for m in targets}
    rho = np.empty((npen, nx))
    near = 0
    for i in range(npen):
        rho[i] = pencil(nx, j0, t_of[int(targets[i % len(targets)])] * (1 + d[i]))
        arg = lad_argument(chi_max(window(rho[i], j0 - 1)))
        near += abs(arg - round(arg)) < 5e-4
    return rho.reshape(nz, ny, nx), int(near)


def teno_field(nx, ny, nz):
    """rho pencils along x whose TENO (cut-off 1e-6) minimum quotient at the
    face before the jump (right-going side) lies within a spread of the
    cut-off.  The flux reconstructs characteristic values that are affine in
    rho for an entropy wave, which leaves the quotients unchanged up to the
    scaled epsilon; the spread covers that shift."""
    npen = ny * nz
    j0 = nx // 4
    qmin = lambda w: float(quotients(w, 0.0)[0].min())
    t_star = crossing_t(nx, j0, 1e-6, qmin)
    d = spread(npen, 1e-10, 1e-2)
    rho = np.stack([pencil(nx, j0, t_star * (1 + d[i])) for i in range(npen)])
    return rho.reshape(nz, ny, nx)
