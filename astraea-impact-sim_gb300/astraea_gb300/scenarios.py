"""Seeded synthetic initial conditions for the benchmark configurations.

These stand in for the engine's PlanetBuilder scenes (engine/planet_builder.cpp),
which are host-side set-up code outside the per-step path.  Every builder
returns a host particle state (dict field -> numpy array, ParticleBuffersDevice
field names) ready for DeviceParticles.upload.

* two_granite_spheres -- jittered cubic lattice spheres, R 1.0 and 0.6 PSU,
  12,288 + 4,096 particles, uniform Granite at rho0.  Equal particle masses
  and those radii and counts cannot all hold at one density (the volume ratio
  0.216 would need ~2,654 impactor particles), so N and R are kept, both
  bodies are at rho0, and the impactor's particles are 0.648x lighter.
* differentiated_impact -- Iron core (30 % of mass) + Granite mantle bodies
  with the radial density of a 1-D hydrostatic integration (FP64 Tillotson
  cold curve + thermal term at a fixed temperature), target:impactor mass
  10:1, placed on the two-body approach orbit of engine/simulation.cpp:
  1389-1436.
* plummer_sphere -- N equal masses from a Plummer profile (a = 1, G = 1),
  masses scaled by 1/G_PSU so the engine's G_PSU gravity acts like G = 1,
  softening eps = 0.8 h0 = 1e-3.
"""
import math

import numpy as np

from . import abi

G_PSU = 6.67430e-11 * 1.0e24 * 1.0e3 * 1.0e3 / 1.0e18   # engine/units.hpp:21
M_EARTH_PSU = 5.97219e24 / 1.0e24

# Published EOS constants (SI) of Iron (0) and Granite (1) used for the
# hydrostatic profile (the same table the EOS kernels use).
_MAT = {
    0: dict(rho0=7800.0, a=0.5, b=1.5, A=1.28e11, B=1.05e11, E0=9.5e6, cv=449.0, tRef=293.0, epsFailMin=1.0e-3),
    1: dict(rho0=2680.0, a=0.5, b=1.3, A=1.80e10, B=1.80e10, E0=1.6e7, cv=790.0, tRef=293.0, epsFailMin=1.0e-4),
    2: dict(rho0=1000.0, a=0.7, b=0.15, A=2.18e9, B=1.325e10, E0=7.0e6, cv=4184.0, tRef=273.15, epsFailMin=5.0e-4),
    4: dict(rho0=2000.0, a=0.5, b=1.3, A=1.20e10, B=1.20e10, E0=1.6e7, cv=800.0, tRef=293.0, epsFailMin=5.0e-5),
}


def empty_state(n):
    st = {name: np.zeros(n, dtype=dt) for name, dt in abi.FIELDS}
    st["tracerIndex"][:] = -1
    st["shepardC"][:] = 1.0
    return st


def cold_energy_si(mat, rho):
    """u_cold(rho) in J/kg (cold compression integral of the Tillotson curve)."""
    p = _MAT[mat]
    eta = np.maximum(np.asarray(rho, dtype=np.float64) / p["rho0"], 1.0)
    mu = eta - 1.0
    le = np.log1p(mu)
    ta = le - mu / eta
    tb = mu * (2.0 + mu) / eta - 2.0 * le
    return (p["A"] * ta + p["B"] * tb) / p["rho0"]


def pressure_si(mat, rho, temp):
    """Tillotson compressed-branch pressure (Pa) at density rho and temperature T."""
    p = _MAT[mat]
    rho = np.asarray(rho, dtype=np.float64)
    eta = rho / p["rho0"]
    mu = eta - 1.0
    uc = cold_energy_si(mat, rho)
    ue = uc + np.maximum(0.0, p["cv"] * (temp - p["tRef"]))
    w = ue / (p["E0"] * eta * eta) + 1.0
    bEff = np.where(mu >= 0.0, p["B"], 0.0)
    return (p["a"] + p["b"] / w) * rho * ue + p["A"] * mu + bEff * mu * mu


def density_at(mat, P, temp):
    """Invert pressure_si for rho >= rho0 by bisection (vectorised)."""
    p = _MAT[mat]
    lo = np.full_like(np.asarray(P, dtype=np.float64), p["rho0"])
    hi = lo * 8.0
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        f = pressure_si(mat, mid, temp) - P
        hi = np.where(f > 0.0, mid, hi)
        lo = np.where(f > 0.0, lo, mid)
    return 0.5 * (lo + hi)


def _rho_of_p_table(mat, temp):
    """rho(P) at fixed T on a log grid of pressures (Pa), for interpolation."""
    P = np.concatenate([[0.0], np.logspace(4.0, 13.5, 3000)])
    return P.tolist(), density_at(mat, P, temp).tolist()


def hydrostatic_profile(mass_psu, core_frac, temp=2000.0, samples=3000):
    """Radial profile (r [m], m(r) [kg], rho [kg/m^3], material) of an
    Iron-core + Granite body in hydrostatic equilibrium, by shooting on the
    central pressure: dm/dr = 4 pi r^2 rho, dP/dr = -G m rho / r^2, with rho
    from the EOS at temperature `temp`."""
    import bisect
    M = mass_psu * 1.0e24
    G = 6.67430e-11
    tables = {m: _rho_of_p_table(m, temp) for m in (0, 1)}

    def rho_at(mat, P):
        Ps, rs = tables[mat]
        if P <= 0.0:
            return rs[0]
        k = bisect.bisect_right(Ps, P)
        if k >= len(Ps):
            return rs[-1]
        t = (P - Ps[k - 1]) / (Ps[k] - Ps[k - 1])
        return rs[k - 1] + t * (rs[k] - rs[k - 1])

    r_est = (3.0 * M / (4.0 * math.pi * 5000.0)) ** (1.0 / 3.0)
    dr = 1.5 * r_est / samples

    def integrate(pc, record):
        r, m, P = 0.0, 0.0, pc
        mat = 0 if core_frac > 0 else 1
        out = ([0.0], [0.0], [rho_at(mat, P)], [mat]) if record else None
        while P > 0.0 and m < 1.5 * M:
            if mat == 0 and m >= core_frac * M:
                mat = 1
            rho = rho_at(mat, P)
            rm = r + 0.5 * dr
            dm = 4.0 * math.pi * rm * rm * rho * dr
            dP = -G * (m + 0.5 * dm) * rho / (rm * rm) * dr if rm > 0 else 0.0
            r += dr
            m += dm
            P += dP
            if record:
                out[0].append(r); out[1].append(m); out[2].append(rho); out[3].append(mat)
        return m, out

    lo, hi = 1.0e8, 3.0e13
    for _ in range(48):
        pc = math.sqrt(lo * hi)
        m, _ = integrate(pc, False)
        if m > M:
            hi = pc
        else:
            lo = pc
    _, out = integrate(math.sqrt(lo * hi), True)
    rs, ms, rhos, mats = (np.array(v) for v in out)
    ms *= M / ms[-1]          # close the residual mass error of the shooting
    return rs, ms, rhos, mats


def _lattice_ball(n, rng, jitter=0.1):
    """n points of a jittered cubic lattice filling a unit ball (radius 1)."""
    s = (4.0 / 3.0 * math.pi / n) ** (1.0 / 3.0)
    k = int(math.ceil(1.0 / s)) + 2
    ax = (np.arange(-k, k + 1) + 0.5) * s
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    r = np.linalg.norm(pts, axis=1)
    order = np.argsort(r, kind="stable")
    pts = pts[order[:n]]
    pts /= max(np.linalg.norm(pts, axis=1).max() + 0.5 * s, 1e-12)
    pts += rng.uniform(-jitter, jitter, size=pts.shape) * s
    return pts, s


def shell_ball(n, rng):
    """n points on concentric Fibonacci-spiral shells filling a unit ball,
    one shell per mean particle spacing, each shell randomly rotated; the
    outermost shell lies half a spacing inside the surface."""
    s = (4.0 / 3.0 * math.pi / n) ** (1.0 / 3.0)
    nsh = max(1, int(round(1.0 / s)))
    radii = (np.arange(nsh) + 0.5) / nsh
    w = radii ** 2
    counts = np.floor(n * w / w.sum()).astype(int)
    counts[np.argsort(-(n * w / w.sum() - counts))[: n - counts.sum()]] += 1
    golden = math.pi * (3.0 - math.sqrt(5.0))
    out = []
    for r, c in zip(radii, counts):
        if c == 0:
            continue
        k = np.arange(c)
        zz = 1.0 - 2.0 * (k + 0.5) / c
        rxy = np.sqrt(np.maximum(0.0, 1.0 - zz * zz))
        th = golden * k
        v = np.stack([rxy * np.cos(th), rxy * np.sin(th), zz], 1)
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        out.append(r * v @ q.T)
    return np.concatenate(out)[:n]


def _weibull_eps(rng, n, eps_min):
    w = -np.log(rng.uniform(1e-6, 1.0 - 1e-6, size=n))
    return (eps_min * np.clip(np.maximum(w, 1e-6) ** (1.0 / 9.0), 1.0, 3.0)).astype(np.float32)


def _uniform_body(n, radius, mat, temp, body_id, rng, shells=False):
    p = _MAT[mat]
    rho = p["rho0"] / 1.0e6
    pts = shell_ball(n, rng) if shells else _lattice_ball(n, rng)[0]
    pts *= radius
    m = rho * 4.0 / 3.0 * math.pi * radius ** 3 / n
    h0 = 1.2 * (m / rho) ** (1.0 / 3.0)
    st = empty_state(n)
    st["posX"][:], st["posY"][:], st["posZ"][:] = pts[:, 0], pts[:, 1], pts[:, 2]
    st["mass"][:] = m
    st["h"][:] = h0
    st["h0"][:] = h0
    st["rho"][:] = rho
    st["u"][:] = (p["cv"] * temp) / 1.0e6
    st["tempK"][:] = temp
    st["epsFail"][:] = _weibull_eps(rng, n, p["epsFailMin"])
    st["materialId"][:] = mat
    st["bodyId"][:] = body_id
    return st


def _layered_body(n, mass_psu, core_frac, temp, body_id, rng):
    rs, ms, rhos, mats = hydrostatic_profile(mass_psu, core_frac, temp)
    M = ms[-1]
    pts, _ = _lattice_ball(n, rng)
    r0 = np.linalg.norm(pts, axis=1)
    frac = np.clip(r0, 0.0, 1.0) ** 3                  # enclosed-mass fraction of a uniform ball
    # equal-mass particles: radius where m(r)/M matches the lattice fraction
    r = np.interp(frac * M, ms, rs)
    scale = np.where(r0 > 0, r / np.maximum(r0, 1e-30), 0.0)
    pts = pts * scale[:, None] / 1.0e6                 # metres -> PSU
    rho = np.interp(r, rs, rhos) / 1.0e6
    mat = np.where(frac * M < core_frac * M, 0, 1).astype(np.uint8)
    m = mass_psu / n
    st = empty_state(n)
    st["posX"][:], st["posY"][:], st["posZ"][:] = pts[:, 0], pts[:, 1], pts[:, 2]
    st["mass"][:] = m
    h0 = 1.2 * (m / rho) ** (1.0 / 3.0)
    st["h"][:] = h0
    st["h0"][:] = h0
    st["rho"][:] = rho
    uc = np.where(mat == 0, cold_energy_si(0, rho * 1e6), cold_energy_si(1, rho * 1e6))
    cv = np.where(mat == 0, _MAT[0]["cv"], _MAT[1]["cv"])
    st["u"][:] = (uc + cv * temp) / 1.0e6
    st["tempK"][:] = temp
    eps = np.where(mat == 0, _weibull_eps(rng, n, _MAT[0]["epsFailMin"]), _weibull_eps(rng, n, _MAT[1]["epsFailMin"]))
    st["epsFail"][:] = eps
    st["materialId"][:] = mat
    st["bodyId"][:] = body_id
    return st, float(rs[-1] / 1.0e6)


def _merge_on_orbit(t, i, r_t, r_i, v_ratio, b, sep_radii):
    """Two-body approach orbit in the COM frame (engine/simulation.cpp:1389-1436)."""
    mt = float(np.sum(t["mass"], dtype=np.float64))
    mi = float(np.sum(i["mass"], dtype=np.float64))
    mtot = mt + mi
    rc = max(r_t + r_i, 1.0e-3)
    v_esc = math.sqrt(2.0 * G_PSU * mtot / rc)
    vc = max(0.0, v_ratio) * v_esc
    d0 = max(sep_radii, 1.0) * rc
    v0sq = vc * vc - 2.0 * G_PSU * mtot * (1.0 / rc - 1.0 / d0)
    if v0sq < 0.0:
        r_apo = rc / max(1.0 - v_ratio * v_ratio, 1.0e-6)
        d0 = min(max(0.98 * r_apo, 1.01 * rc), d0)
        v0sq = max(0.0, vc * vc - 2.0 * G_PSU * mtot * (1.0 / rc - 1.0 / d0))
    v0 = math.sqrt(v0sq)
    b = max(-1.2, min(1.2, b))
    v_perp = rc * vc * b / d0
    if abs(v_perp) > 0.995 * v0:
        v_perp = math.copysign(0.995 * v0, v_perp)
    v_rad = -math.sqrt(max(0.0, v0 * v0 - v_perp * v_perp))
    ft, fi = -mi / mtot, mt / mtot
    for st, f in ((t, ft), (i, fi)):
        st["posX"] += np.float32(f * d0)
        st["velX"] += np.float32(f * v_rad)
        st["velZ"] += np.float32(f * (-v_perp))
    out = {k: np.concatenate([t[k], i[k]]) for k in t}
    out["originalId"] = np.arange(len(out["posX"]), dtype=np.uint32)
    out["velHalfX"], out["velHalfY"], out["velHalfZ"] = out["velX"].copy(), out["velY"].copy(), out["velZ"].copy()
    return out, dict(v_esc=v_esc, r_contact=rc, d0=d0, m_target=mt, m_impactor=mi)


def two_granite_spheres(n_target=12288, n_impactor=4096, r_target=1.0, r_impactor=0.6, v_ratio=1.1,
                        angle_deg=45.0, sep_radii=1.02, temp=300.0, seed=42):
    rng = np.random.Generator(np.random.PCG64(seed))
    t = _uniform_body(n_target, r_target, 1, temp, 0, rng)
    i = _uniform_body(n_impactor, r_impactor, 1, temp, 1, rng)
    return _merge_on_orbit(t, i, r_target, r_impactor, v_ratio, math.sin(math.radians(angle_deg)), sep_radii)


def differentiated_impact(n_total=1_000_000, impactor_frac=0.2, mass_target=M_EARTH_PSU, mass_ratio=0.1,
                          core_frac=0.3, v_ratio=1.1, angle_deg=45.0, sep_radii=1.05, temp=2000.0, seed=42):
    rng = np.random.Generator(np.random.PCG64(seed))
    n_i = int(round(n_total * impactor_frac))
    n_t = n_total - n_i
    t, r_t = _layered_body(n_t, mass_target, core_frac, temp, 0, rng)
    i, r_i = _layered_body(n_i, mass_target * mass_ratio, core_frac, temp, 1, rng)
    return _merge_on_orbit(t, i, r_t, r_i, v_ratio, math.sin(math.radians(angle_deg)), sep_radii)


def _polytrope_envelope(n, mass_psu, r_in, r_out, temp, body_id, rng):
    """HydrogenHelium (material 3) shell r_in..r_out with the n = 1 polytrope
    profile rho ~ sin(pi r / r_out) / (pi r / r_out), equal-mass particles."""
    rs = np.linspace(r_in, r_out, 4000)
    x = np.pi * rs / r_out
    shape = np.sin(x) / x
    dm = 4.0 * np.pi * rs * rs * shape
    ms = np.concatenate([[0.0], np.cumsum(0.5 * (dm[1:] + dm[:-1]) * np.diff(rs))])
    rho_c = mass_psu / ms[-1]
    pts, _ = _lattice_ball(n, rng)
    r0 = np.linalg.norm(pts, axis=1)
    frac = np.clip(r0, 0.0, 1.0) ** 3
    r = np.interp(frac * ms[-1], ms, rs)
    scale = np.where(r0 > 0, r / np.maximum(r0, 1e-30), 0.0)
    pts = pts * scale[:, None]
    rho = np.maximum(rho_c * np.interp(r, rs, shape), 1.0e-9)
    m = mass_psu / n
    st = empty_state(n)
    st["posX"][:], st["posY"][:], st["posZ"][:] = pts[:, 0], pts[:, 1], pts[:, 2]
    st["mass"][:] = m
    h0 = 1.2 * (m / rho) ** (1.0 / 3.0)
    st["h"][:] = h0
    st["h0"][:] = h0
    st["rho"][:] = rho
    st["u"][:] = (8260.0 * temp) / 1.0e6          # HydrogenHelium c_v, thermal part
    st["tempK"][:] = temp
    st["epsFail"][:] = 1.0
    st["materialId"][:] = 3
    st["bodyId"][:] = body_id
    return st


def gas_giant_impact(n_total=16_000_000, n_impactor=2_000_000, mass_target=10.0 * M_EARTH_PSU, core_mass_frac=0.1,
                     envelope_radius_factor=4.0, mass_ratio=0.1, v_ratio=2.0, angle_deg=30.0, temp=2000.0, seed=42):
    """Gas-giant core impact: a HydrogenHelium n = 1 polytrope envelope over an
    Iron + Granite core holding core_mass_frac of the target mass, hit by a
    uniform Regolith impactor.  Particle counts split by mass between core and
    envelope (equal particle mass within each)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n_t = n_total - n_impactor
    n_core = max(1024, int(round(n_t * core_mass_frac)))
    core, r_core = _layered_body(n_core, mass_target * core_mass_frac, 0.33, temp, 0, rng)
    env = _polytrope_envelope(n_t - n_core, mass_target * (1.0 - core_mass_frac), r_core,
                              envelope_radius_factor * r_core, temp, 0, rng)
    target = {k: np.concatenate([core[k], env[k]]) for k in core}
    m_i = mass_target * mass_ratio
    rho_i = 2000.0 / 1.0e6
    r_i = (3.0 * m_i / (4.0 * math.pi * rho_i)) ** (1.0 / 3.0)
    imp = _uniform_body(n_impactor, r_i, 4, temp, 1, rng)
    imp["mass"][:] = m_i / n_impactor
    return _merge_on_orbit(target, imp, envelope_radius_factor * r_core, r_i, v_ratio,
                           math.sin(math.radians(angle_deg)), 1.05)


def ensemble_impact(n_total, material=1, v_ratio=1.1, angle_deg=45.0, r_target=1.0, r_impactor=0.6, temp=300.0,
                    seed=42):
    """Two uniform single-material spheres (radii 1.0 and 0.6, equal density,
    particles split by volume) on the impact orbit of _merge_on_orbit."""
    rng = np.random.Generator(np.random.PCG64(seed))
    vol_i = r_impactor ** 3 / (r_target ** 3 + r_impactor ** 3)
    n_i = max(64, int(round(n_total * vol_i)))
    t = _uniform_body(n_total - n_i, r_target, material, temp, 0, rng)
    i = _uniform_body(n_i, r_impactor, material, temp, 1, rng)
    return _merge_on_orbit(t, i, r_target, r_impactor, v_ratio, math.sin(math.radians(angle_deg)), 1.05)


def ensemble_configs(count=64, n_min=8192, n_max=131072, seed=7):
    """Instances of the batched-ensemble workload: N log-uniform in
    [n_min, n_max], impact angle uniform in 0..75 deg, velocity uniform in
    1..3 v_esc, material drawn from Iron, Granite, WaterIce, Regolith."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(count):
        out.append(dict(n_total=int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))),
                        material=int(rng.choice([0, 1, 2, 4])), v_ratio=float(rng.uniform(1.0, 3.0)),
                        angle_deg=float(rng.uniform(0.0, 75.0)), seed=int(seed * 1000 + k)))
    return out


def plummer_sphere(n, a=1.0, softening=1.0e-3, seed=42):
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.uniform(1e-10, 1.0 - 1e-10, size=n)
    r = a / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
    r = np.minimum(r, 100.0 * a)
    cth = rng.uniform(-1.0, 1.0, size=n)
    phi = rng.uniform(0.0, 2.0 * math.pi, size=n)
    sth = np.sqrt(1.0 - cth * cth)
    st = empty_state(n)
    st["posX"][:] = r * sth * np.cos(phi)
    st["posY"][:] = r * sth * np.sin(phi)
    st["posZ"][:] = r * cth
    st["mass"][:] = (1.0 / n) / G_PSU
    h0 = softening / 0.8
    st["h"][:] = h0
    st["h0"][:] = h0
    st["rho"][:] = 1.0e-3
    st["materialId"][:] = 1
    st["originalId"][:] = np.arange(n, dtype=np.uint32)
    return st
