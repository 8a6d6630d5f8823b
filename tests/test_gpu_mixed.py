"""The mixed-precision form (FP32 momentum, compensated-FP32 ssh) against
the FP64 path, which the parity tests pin bit for bit to the reference.
Bar (stated per field): ssh RMS error <= 1e-6 m after 1000 steps on a
seeded Fourier bathymetry."""
import numpy as np
import pytest

import nl2d_testlib as T

pytestmark = pytest.mark.gpu


def bathy_model(n, seed, oracle):
    from psyclonebench_gb300.workloads import fourier_depth
    m = T.make_model(n + 2, n + 2, 1, width=((n + 3 + 7) // 8) * 8, oracle=oracle)
    ht, hu, hv = fourier_depth(m.width, m.height, seed)
    m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = ht, hu, hv
    m.rdt = 5.0  # gravity-wave CFL at 500 m depth (sqrt(g h) = 70 m/s, dx = 1 km)
    return m


def run_form(gpulib, m, nsteps, precision):
    import psyclonebench_gb300 as P
    T.gpu_register(gpulib, m)
    gpulib.nl2d_set_precision(precision)
    out = np.zeros(3)
    P.check(gpulib.nl2d_run_steps(1, nsteps, 0, T.dptr(out)), "run")
    T.gpu_read_all(gpulib, m)
    gpulib.nl2d_set_precision(0)
    return m


def test_mixed_error_vs_fp64(gpulib, oracle):
    base = bathy_model(256, 42, oracle)
    ref = run_form(gpulib, base.copy(), 1000, 0)
    mix = run_form(gpulib, base.copy(), 1000, 1)
    assert gpulib.nl2d_last_path() in (3, 0)
    report = {}
    for k, (x0, x1, y0, y1) in (("sshn_t", T.regions(ref)["t"]), ("un", T.regions(ref)["u"]),
                                ("vn", T.regions(ref)["v"])):
        a = mix.f[k][y0:y1 + 1, x0:x1 + 1]
        b = ref.f[k][y0:y1 + 1, x0:x1 + 1]
        report[k] = (float(np.sqrt(np.mean((a - b) ** 2))), float(np.abs(a - b).max()),
                     float(np.abs(b).max()))
    print("mixed vs fp64 after 1000 steps (rms, max, field max):", report)
    assert report["sshn_t"][0] <= 1e-6
    assert report["un"][0] <= 1e-4 * report["un"][2]
    assert report["vn"][0] <= 1e-4 * report["vn"][2]


def test_mixed_error_vs_fp64_4096(gpulib, oracle):
    """The benchmark's own size (4096^2 interior, config 2's bathymetry):
    after 500 steps the mixed state's ssh RMS error against the FP64 path
    stays within 1e-6 m and u, v within 1e-4 of their largest value."""
    base = bathy_model(4096, 2, oracle)
    ref = run_form(gpulib, base.copy(), 500, 0)
    mix = run_form(gpulib, base, 500, 1)
    report = {}
    for k, (x0, x1, y0, y1) in (("sshn_t", T.regions(ref)["t"]), ("un", T.regions(ref)["u"]),
                                ("vn", T.regions(ref)["v"])):
        a = mix.f[k][y0:y1 + 1, x0:x1 + 1]
        b = ref.f[k][y0:y1 + 1, x0:x1 + 1]
        assert np.isfinite(a).all(), k
        report[k] = (float(np.sqrt(np.mean((a - b) ** 2))), float(np.abs(b).max()))
    print("mixed vs fp64 at 4096^2 after 500 steps (rms, field max):", report)
    assert report["sshn_t"][0] <= 1e-6
    assert report["un"][0] <= 1e-4 * report["un"][1]
    assert report["vn"][0] <= 1e-4 * report["vn"][1]


def test_mixed_nonzero_ssha_uv_vs_fp64(gpulib, oracle):
    """With ssha_u and ssha_v nonzero (1 m and 0.5 m on 50-500 m depths) the
    march must read the stored reciprocals 1 / (hu + ssha_u), 1 / (hv +
    ssha_v) rather than form them from the depths alone (an error of about
    1 % in u and v): the same bars against the FP64 path hold."""
    base = bathy_model(192, 5, oracle)
    base.f["ssha_u"][:] = 1.0
    base.f["ssha_v"][:] = 0.5
    ref = run_form(gpulib, base.copy(), 300, 0)
    mix = run_form(gpulib, base, 300, 1)
    for k, reg, bar in (("sshn_t", "t", None), ("un", "u", 1e-4), ("vn", "v", 1e-4)):
        x0, x1, y0, y1 = T.regions(ref)[reg]
        a = mix.f[k][y0:y1 + 1, x0:x1 + 1]
        b = ref.f[k][y0:y1 + 1, x0:x1 + 1]
        rms = float(np.sqrt(np.mean((a - b) ** 2)))
        assert rms <= (1e-6 if bar is None else bar * float(np.abs(b).max())), (k, rms)


def test_mixed_checksums_and_roundtrip(gpulib, oracle):
    """In-graph checksums of the mixed state agree with the FP64 image that
    c_read_from_device returns, and switching back to FP64 continues."""
    import psyclonebench_gb300 as P
    m = bathy_model(64, 3, oracle)
    T.gpu_register(gpulib, m)
    gpulib.nl2d_set_precision(1)
    sums = np.zeros(6)
    P.check(gpulib.nl2d_run_steps(1, 100, 50, T.dptr(sums)), "run mixed")
    T.gpu_read_all(gpulib, m)
    cs = T.model_checksums(m, oracle)
    np.testing.assert_allclose(sums[3:], [cs["sshn_t"], cs["un"], cs["vn"]], rtol=1e-10)
    gpulib.nl2d_set_precision(0)
    P.check(gpulib.nl2d_run_steps(101, 20, 0, T.dptr(sums)), "run fp64 after mixed")
    T.gpu_read_all(gpulib, m)
    assert np.isfinite(m.f["sshn_t"]).all()


def test_mixed_random_land_vs_fp64(gpulib, oracle):
    """8 % random land cells inside a bathymetry domain: the cells next to
    land are updated by the mixed step's general path (the column march
    leaves them out), the rest by the march; after 300 steps the mixed
    fields stay within the same bar against FP64."""
    rng = np.random.default_rng(4)
    base = bathy_model(192, 7, oracle)
    inner = base.grid["tmask"][base.ys + 1:base.ye, base.xs + 1:base.xe]
    inner[rng.random(inner.shape) < 0.08] = 0
    ref = run_form(gpulib, base.copy(), 300, 0)
    mix = run_form(gpulib, base.copy(), 300, 1)
    report = {}
    for k, (x0, x1, y0, y1) in (("sshn_t", T.regions(ref)["t"]), ("un", T.regions(ref)["u"]),
                                ("vn", T.regions(ref)["v"])):
        a = mix.f[k][y0:y1 + 1, x0:x1 + 1]
        b = ref.f[k][y0:y1 + 1, x0:x1 + 1]
        assert np.isfinite(a).all(), k
        report[k] = (float(np.sqrt(np.mean((a - b) ** 2))), float(np.abs(a - b).max()),
                     float(np.abs(b).max()))
    print("mixed vs fp64 with land, 300 steps (rms, max, field max):", report)
    assert report["sshn_t"][0] <= 1e-6
    assert report["un"][0] <= 1e-4 * report["un"][2]
    assert report["vn"][0] <= 1e-4 * report["vn"][2]


@pytest.mark.parametrize("jphgr,nx,ny", [(2, 97, 61), (3, 75, 130)])
def test_mixed_other_masks_vs_fp64(gpulib, oracle, jphgr, nx, ny):
    """The T masks of jphgr_msh 2 and 3 (model_mod.f90:94-249) on odd-sized
    grids with a padded width: the column march and its general pass against
    FP64 after 300 steps, same bar."""
    from psyclonebench_gb300.workloads import fourier_depth
    m = T.make_model(nx + 2, ny + 2, jphgr, width=nx + 9, oracle=oracle)
    ht, hu, hv = fourier_depth(m.width, m.height, 5)
    m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = ht, hu, hv
    m.rdt = 5.0
    ref = run_form(gpulib, m.copy(), 300, 0)
    mix = run_form(gpulib, m.copy(), 300, 1)
    assert gpulib.nl2d_last_path() in (3, 0)  # the mixed form ran
    for k, (x0, x1, y0, y1) in (("sshn_t", T.regions(ref)["t"]), ("un", T.regions(ref)["u"]),
                                ("vn", T.regions(ref)["v"])):
        a = mix.f[k][y0:y1 + 1, x0:x1 + 1]
        b = ref.f[k][y0:y1 + 1, x0:x1 + 1]
        assert np.isfinite(a).all(), k
        rms = float(np.sqrt(np.mean((a - b) ** 2)))
        if k == "sshn_t":
            assert rms <= 1e-6, (k, rms)
        else:
            assert rms <= 1e-4 * max(float(np.abs(b).max()), 1e-12), (k, rms)
