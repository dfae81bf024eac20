"""Seeded synthetic scenes for the five benchmark configurations.

The reference publishes no dataset; scenes are drawn here from counter-based
generators (numpy Philox) with fixed seeds, with the shapes and value
distributions of the benchmark configurations:

  1 plain    one sphere a = 5 um, n = 1.4 + 0.05i at the origin, lambda 2.5 um,
             condenser/objective NA 0-0.5, 400 waves, 256^2 over 20 um,
             --padding 2, direct (recursive) evaluation, field order 10
  2 headline 1024^2 over 100 um, 50 non-overlapping spheres at z = 0,
             a ~ U(1, 5), n ~ U(1.2, 1.6) + i U(0, 0.05), lambda 3 um,
             1000 waves, scalar LUT mode + incident-field LUT,
             LUTs of 4096 radial x 1024 angular samples
  3 sweep    config 2 scene at 512^2 over 512 wavelengths in 2.5-12.5 um
  5 large    4096^2 over 400 um, 1000 spheres a ~ U(2, 20) in a slab
             |z| < 60 um, lambda 2 um, 2000 waves
"""
import math

import numpy as np

from . import abi


def rng(seed):
    return np.random.Generator(np.random.Philox(seed))


def mc_waves(nk, na_in=0.0, na_out=0.5, seed=1, kdir=(0.0, 0.0, 1.0)):
    """Directions uniform on the condenser annulus, as mcSampleNA draws them
    (montecarlo.cpp:9-71): cos(polar) uniform between cos(asin NA_out) and
    cos(asin NA_in), azimuth uniform, rotated from +z onto kdir."""
    g = rng(seed)
    zin, zout = math.cos(math.asin(na_in)), math.cos(math.asin(na_out))
    z = g.uniform(0.0, 1.0, nk) * (zin - zout) + zout
    az = g.uniform(0.0, 2 * math.pi, nk)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    v = np.stack([np.cos(az) * s, np.sin(az) * s, z], axis=1)
    k = np.asarray(kdir, dtype=np.float64)
    k = k / np.linalg.norm(k)
    c = k[2]
    if c < 1.0 - 1e-15:
        axis = np.cross([0.0, 0.0, 1.0], k)
        axis /= np.linalg.norm(axis)
        ang = math.acos(max(-1.0, min(1.0, c)))
        K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
        Rm = np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * (K @ K)
        v = v @ Rm.T
    return np.ascontiguousarray(v)


def random_spheres(n, fov, a_lo, a_hi, nre=(1.2, 1.6), nim=(0.0, 0.05), seed=2, z_slab=0.0, max_tries=200000):
    """Non-overlapping spheres with centres uniform in the field of view
    (z = 0, or uniform in |z| < z_slab), radii uniform in [a_lo, a_hi]."""
    g = rng(seed)
    out = []
    tries = 0
    while len(out) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place spheres without overlap")
        a = g.uniform(a_lo, a_hi)
        x, y = g.uniform(-fov / 2, fov / 2, 2)
        z = g.uniform(-z_slab, z_slab) if z_slab > 0 else 0.0
        ok = all((x - s[0]) ** 2 + (y - s[1]) ** 2 + (z - s[2]) ** 2 > (a + s[3]) ** 2 for s in out)
        if ok:
            out.append((x, y, z, a, g.uniform(*nre), g.uniform(*nim)))
    return out


def config1(resolution=256):
    """Plain method: direct evaluation, one sphere at the origin."""
    p = abi.make_params(lam=2.5, condenser=(0.0, 0.5), objective=(0.0, 0.5), xy=(20.0, 0.0),
                        resolution=resolution, padding=2, field_order=10, lut_us=False, lut_uf=False)
    spheres = [(0.0, 0.0, 0.0, 5.0, 1.4, 0.05)]
    return p, spheres, mc_waves(400, 0.0, 0.5, seed=1)


def config2(resolution=1024, fov=100.0, n_spheres=50, samples=1000, lut_r=4096, lut_theta=1024, seed=2):
    """Headline scene: scalar LUT mode plus incident-field LUT."""
    p = abi.make_params(lam=3.0, condenser=(0.0, 0.5), objective=(0.0, 0.5), xy=(fov, 0.0),
                        resolution=resolution, padding=1, field_order=10, lut_us=True, lut_uf=True,
                        us_lut_r=lut_r, us_lut_theta=lut_theta, uf_lut_r=lut_r)
    spheres = random_spheres(n_spheres, fov, 1.0, 5.0, seed=seed)
    return p, spheres, mc_waves(samples, 0.0, 0.5, seed=seed)


def config5(resolution=4096, n_spheres=1000, samples=2000):
    p = abi.make_params(lam=2.0, condenser=(0.0, 0.5), objective=(0.0, 0.5), xy=(400.0, 0.0),
                        resolution=resolution, padding=1, field_order=10, lut_us=True, lut_uf=True,
                        us_lut_r=4096, us_lut_theta=1024, uf_lut_r=4096)
    spheres = random_spheres(n_spheres, 400.0, 2.0, 20.0, seed=5, z_slab=60.0)
    return p, spheres, mc_waves(samples, 0.0, 0.5, seed=5)


def served_trace(n, seed=4, resolutions=(128, 256, 512, 1024, 2048), rate_hz=1.0, repeat_frac=0.25):
    """Requests of the served workload: Poisson arrivals at rate_hz, res from
    `resolutions`, S ~ U{1..200} spheres as in config 2 (100 um field, a ~ U(1, 5),
    n ~ U(1.2, 1.6) + i U(0, 0.05); a slab |z| < 30 um once the plane is too
    crowded), lambda ~ U(2.5, 12.5) um, nk from {200, 1000, 2000}, LUTs of 4096 x
    1024; a fraction repeat_frac of the requests re-images an earlier scene
    with new directions.  Returns [(t_arrival_s, params, spheres, waves)]."""
    g = rng(seed)
    out = []
    t = 0.0
    for i in range(n):
        t += g.exponential(1.0 / rate_hz)
        if out and g.uniform() < repeat_frac:
            _, p, s, w = out[int(g.integers(0, len(out)))]
            w = mc_waves(len(w), 0.0, 0.5, seed=seed * 100003 + i)
            out.append((t, p, s, w))
            continue
        res = int(g.choice(resolutions))
        ns = int(g.integers(1, 201))
        lam = float(g.uniform(2.5, 12.5))
        nk = int(g.choice([200, 1000, 2000]))
        p = abi.make_params(lam=lam, condenser=(0.0, 0.5), objective=(0.0, 0.5), xy=(100.0, 0.0),
                            resolution=res, padding=1, field_order=10, lut_us=True, lut_uf=True,
                            us_lut_r=4096, us_lut_theta=1024, uf_lut_r=4096)
        s = random_spheres(ns, 100.0, 1.0, 5.0, seed=seed * 1009 + i, z_slab=0.0 if ns <= 60 else 30.0)
        out.append((t, p, s, mc_waves(nk, 0.0, 0.5, seed=seed * 7919 + i)))
    return out


def lorentz_kappa(nu, centres_um, widths_um, peaks):
    """Absorption index: Lorentzian bands in wavenumber nu (1/um), each centred
    at 1/centre with half width (width/2)/centre^2 (so FWHM ~ width in
    wavelength) and the given peak."""
    nu = np.asarray(nu, dtype=np.float64)
    k = np.zeros_like(nu)
    for c, w, pk in zip(centres_um, widths_um, peaks):
        nc, g = 1.0 / c, 0.5 * w / (c * c)
        k += pk * g * g / ((nu - nc) ** 2 + g * g)
    return k


def hilbert_dn(nu_grid, kappa):
    """Kramers-Kronig refractive-index change of an absorption band on a
    uniform wavenumber grid: dn = -H[kappa], H the discrete Hilbert transform
    (FFT, response -i sign(f), zero-padded 4x against wrap-around).  For a
    Lorentzian kappa = p g^2 / ((nu - nc)^2 + g^2) this is
    -p g (nu - nc) / ((nu - nc)^2 + g^2): normal dispersion below the band."""
    n = len(kappa)
    m = 4 * n
    f = np.fft.fft(np.concatenate([kappa, np.zeros(m - n)]))
    freq = np.fft.fftfreq(m)
    h = np.real(np.fft.ifft(-1j * np.sign(freq) * f))[:n]
    return -h


def lorentz_material(lambdas, seed=3, n0=1.45, bands=3):
    """n(lambda) = n0 + dn(lambda) + i kappa(lambda) with `bands` seeded
    Lorentzian absorption bands (centres in 2.5-12.5 um, widths 0.05-0.2 um,
    peaks <= 0.1) and dn from the discrete Hilbert transform of kappa."""
    g = rng(seed)
    centres = g.uniform(2.5, 12.5, bands)
    widths = g.uniform(0.05, 0.2, bands)
    peaks = g.uniform(0.02, 0.1, bands)
    nu_grid = np.linspace(1.0 / 40.0, 1.0 / 1.0, 1 << 16)
    kap = lorentz_kappa(nu_grid, centres, widths, peaks)
    dn = hilbert_dn(nu_grid, kap)
    nu = 1.0 / np.asarray(lambdas, dtype=np.float64)
    return n0 + np.interp(nu, nu_grid, dn) + 1j * lorentz_kappa(nu, centres, widths, peaks)


def config3(n_lambda=512, resolution=512, n_spheres=50, samples=1000, n_materials=3):
    """Spectral sweep: the config-2 scene family at `resolution` over 512
    wavelengths evenly spaced in 2.5-12.5 um; sphere i is made of material
    i % n_materials, each a lorentz_material with its own seed.  Returns
    (params, spheres, waves, lambdas, n_table[n_lambda, n_spheres])."""
    p, spheres, waves = config2(resolution=resolution, n_spheres=n_spheres, samples=samples, seed=3)
    lambdas = np.linspace(2.5, 12.5, n_lambda)
    mats = [lorentz_material(lambdas, seed=30 + j) for j in range(n_materials)]
    table = np.stack([mats[i % n_materials] for i in range(len(spheres))], axis=1)
    return p, spheres, waves, lambdas, table
