"""A second, independent restatement of the tracer-advection iteration
(benchmarks/nemo/tracer_advection/original/tra_adv.F90:107-257), written
with numpy array sections the way the Fortran reads, to cross-check the C
oracle: the reference itself is Fortran and cannot be built here.

Arrays are [jk][jj][ji] (0-based) for the Fortran a(ji, jj, jk); every
operation is one IEEE double operation in the reference's order (numpy does
not contract multiply-adds)."""
import numpy as np


def _max2(a, b):
    return np.where(a > b, a, b)


def _min3(a, b, c):
    m = np.where(a < b, a, b)
    return np.where(m < c, m, c)


def _slope(a, b):
    return (a + b) * (0.25 + np.copysign(0.25, a * b))


def init(jpi, jpj, jpk):
    """tra_adv.F90:63-98."""
    k, j, i = np.meshgrid(np.arange(1, jpk + 1), np.arange(1, jpj + 1), np.arange(1, jpi + 1),
                          indexing="ij")
    v3 = (k * j * i).astype(np.float64) / float(jpi * jpj * jpk)
    j2, i2 = np.meshgrid(np.arange(1, jpj + 1), np.arange(1, jpi + 1), indexing="ij")
    v2 = (j2 * i2).astype(np.float64) / float(jpi * jpj)
    f = {n: v3.copy() for n in ("mydomain", "tsn", "pun", "pvn", "pwn", "umask", "vmask",
                                "tmask")}
    f.update({n: v2.copy() for n in ("ztfreez", "rnfmsk", "upsmsk")})
    f["rnfmsk_z"] = np.array([float(kk // jpk) for kk in range(1, jpk + 1)])
    return f


def step(f, w):
    """One iteration on the dict of inputs f (mydomain updated in place) and
    the dict of persistent work arrays w (zwx, zwy, zslpx, zslpy, zind)."""
    m = f["mydomain"]
    zwx, zwy, zslpx, zslpy, zind = (w[n] for n in ("zwx", "zwy", "zslpx", "zslpy", "zind"))
    K, J, I = m.shape
    zice = np.where(f["tsn"] <= f["ztfreez"][None] + 0.1, 1.0, 0.0)
    mx = _max2(f["rnfmsk"][None] * f["rnfmsk_z"][:, None, None],
               np.broadcast_to(f["upsmsk"][None], m.shape))
    mx = _max2(mx, zice)
    zind[:] = 1 - mx * f["tmask"]

    zwx[K - 1] = 0.0
    zwy[K - 1] = 0.0
    lo = (slice(0, K - 1), slice(0, J - 1), slice(0, I - 1))
    zwx[lo] = f["umask"][lo] * (m[:K - 1, :J - 1, 1:] - m[lo])
    zwy[lo] = f["vmask"][lo] * (m[:K - 1, 1:, :I - 1] - m[lo])

    zslpx[K - 1] = 0.0
    zslpy[K - 1] = 0.0
    up = (slice(0, K - 1), slice(1, J), slice(1, I))
    zslpx[up] = _slope(zwx[up], zwx[:K - 1, 1:, :I - 1])
    zslpy[up] = _slope(zwy[up], zwy[:K - 1, :J - 1, 1:])
    s = zslpx[up].copy()
    zslpx[up] = np.copysign(1.0, s) * _min3(np.abs(s), 2.0 * np.abs(zwx[:K - 1, 1:, :I - 1]),
                                            2.0 * np.abs(zwx[up]))
    s = zslpy[up].copy()
    zslpy[up] = np.copysign(1.0, s) * _min3(np.abs(s), 2.0 * np.abs(zwy[:K - 1, :J - 1, 1:]),
                                            2.0 * np.abs(zwy[up]))

    inn = (slice(0, K - 1), slice(1, J - 1), slice(1, I - 1))
    p = f["pun"][inn]
    z0u = np.copysign(0.5, p)
    zalpha = 0.5 - z0u
    zu = z0u - 0.5 * p * 1.0
    zzwx = m[:K - 1, 1:J - 1, 2:] + zind[inn] * (zu * zslpx[:K - 1, 1:J - 1, 2:])
    zzwy = m[inn] + zind[inn] * (zu * zslpx[inn])
    fx = p * (zalpha * zzwx + (1.0 - zalpha) * zzwy)
    p = f["pvn"][inn]
    z0v = np.copysign(0.5, p)
    zalpha = 0.5 - z0v
    zv = z0v - 0.5 * p * 1.0
    zzwx = m[:K - 1, 2:, 1:I - 1] + zind[inn] * (zv * zslpy[:K - 1, 2:, 1:I - 1])
    zzwy = m[inn] + zind[inn] * (zv * zslpy[inn])
    fy = p * (zalpha * zzwx + (1.0 - zalpha) * zzwy)
    zwx[inn] = fx
    zwy[inn] = fy
    m[inn] = m[inn] + -(1.0 * (zwx[inn] - zwx[:K - 1, 1:J - 1, :I - 2] + zwy[inn] -
                               zwy[:K - 1, :J - 2, 1:I - 1]))

    zwx[0] = 0.0
    zwx[K - 1] = 0.0
    zwx[1:K - 1] = f["tmask"][1:K - 1] * (m[:K - 2] - m[1:K - 1])
    zslpx[0] = 0.0
    zslpx[1:K - 1] = _slope(zwx[1:K - 1], zwx[2:K])
    s = zslpx[1:K - 1].copy()
    zslpx[1:K - 1] = np.copysign(1.0, s) * _min3(np.abs(s), 2.0 * np.abs(zwx[2:K]),
                                                 2.0 * np.abs(zwx[1:K - 1]))
    zwx[0] = f["pwn"][0] * m[0]
    c1 = (slice(1, K), slice(1, J - 1), slice(1, I - 1))
    p1 = f["pwn"][c1]
    z0w = np.copysign(0.5, p1)
    zalpha = 0.5 + z0w
    zw = z0w - 0.5 * p1 * 1.0 * 1.0
    zzwx = m[c1] + zind[inn] * (zw * zslpx[c1])
    zzwy = m[inn] + zind[inn] * (zw * zslpx[inn])
    zwx[c1] = p1 * (zalpha * zzwx + (1.0 - zalpha) * zzwy)
    m[inn] = -(1.0 * (zwx[inn] - zwx[c1]))


def checksum(m):
    """tra_adv.F90:263-270 (in the reference's loop order)."""
    s = 0.0
    K, J, I = m.shape
    for v in m[:K - 1, 1:J - 1, 1:I - 1].reshape(-1):
        s = s + float(v)
    return s
