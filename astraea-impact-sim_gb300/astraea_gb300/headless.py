"""Scenario presets, scenario loading and the conservation check of the
engine's headless runner, on the library's device path.

* PRESETS / preset_config: makePresetConfig (engine/presets.cpp:147-210).
* load_scenario: Simulation::loadScenario (engine/simulation.cpp:1300-1470):
  the particle split between the bodies, each body built on the device
  (astraea_gb300_build_planet) and, with relaxSteps > 0, relaxed on the
  device (astraea_gb300_relax_single_body) between the engine's host-side
  recentring and rigid spin; the two-body Kepler approach orbit, the merge
  with exact system COM and zero net momentum, upload and initial forces.
* run_headless: the step loop and --verify-conservation thresholds of
  engine/headless_main.cpp:169-281 -- fused steps, the device telemetry
  reduction every step, the radiated energy integrated by the trapezoid rule
  (engine/simulation.cpp:1740-1744), energy drift, momentum and angular
  momentum changes normalised as the runner normalises them.
The host-side steps (recentring, spin, orbit placement, merge) act on a
host copy of the bodies, as the engine's do.
"""
import math
import time

import numpy as np
import torch

from . import engine

M_EARTH = 5.97219e24
G_SI = 6.67430e-11
L_UNIT, M_UNIT, T_UNIT = 1.0e6, 1.0e24, 1.0e3
V_UNIT = L_UNIT / T_UNIT
E_UNIT = M_UNIT * V_UNIT * V_UNIT
L_ANG_UNIT = M_UNIT * L_UNIT * V_UNIT
G_PSU = G_SI * M_UNIT * T_UNIT * T_UNIT / (L_UNIT ** 3)

# name: (target archetype, mass, overrides), (impactor archetype, mass, overrides), v/v_esc, b, separation
PRESETS = {
    "EarthTheiaMoonForming": ((0, 1.0 * M_EARTH, {}), (5, 0.13 * M_EARTH, {}), 1.05, 0.72, 3.0),
    "MercuryMantleStrip": ((5, 0.45 * M_EARTH, {"surface_temp_k": 440.0}), (1, 0.22 * M_EARTH, {}), 2.80, 0.35, 3.2),
    "OceanWorldSteamPlume": ((2, 0.75 * M_EARTH, {}), (5, 0.15 * M_EARTH, {}), 1.35, 0.25, 3.2),
    "GasGiantCoreImpact": ((4, 20.0 * M_EARTH, {}), (1, 1.0 * M_EARTH, {}), 1.40, 0.15, 2.8),
    "LivingGaiaAsteroidCataclysm": ((0, 1.0 * M_EARTH, {}),
                                    (5, 0.025 * M_EARTH, {"core_temp_k": 1800.0, "spin": 0.0}), 1.65, 0.30, 3.2),
}


def preset_config(name, total_particles=100000, relax_steps=None):
    """CollisionScenarioConfig of a preset; relax_steps overrides both
    bodies' relaxSteps (the runner's --relax-steps)."""
    (ta, tm, to), (ia, im, io), v, b, sep = PRESETS[name]
    target = engine.body_spec(ta, mass_kg=tm, relax_steps=80, **to)
    impactor = engine.body_spec(ia, mass_kg=im, relax_steps=80, **io)
    if relax_steps is not None:
        target.relaxSteps = impactor.relaxSteps = int(relax_steps)
    return {"name": name, "target": target, "impactor": impactor, "v_ratio": v, "b": b, "sep": sep,
            "total": int(total_particles), "grid": 16, "seed": 42}


BODY_FIELDS = ("posX", "posY", "posZ", "velX", "velY", "velZ", "mass", "h0", "rho", "u", "tempK", "epsFail",
               "materialId", "bodyId", "tracerIndex", "tracerRestRadiusPsu", "tracerRestNormalX",
               "tracerRestNormalY", "tracerRestNormalZ", "tracerIsOcean")


def _center_and_zero_bulk(body):
    """centerAndZeroBulkVelocity (engine/simulation.cpp:298-329)."""
    m = body["mass"].astype(np.float64)
    mt = m.sum()
    if len(m) == 0 or mt <= 0.0:
        return
    for ax in ("posX", "posY", "posZ", "velX", "velY", "velZ"):
        c = np.sum(m * body[ax].astype(np.float64)) / mt
        body[ax] = (body[ax].astype(np.float64) - c).astype(np.float32)


def _apply_spin(body, omega):
    """applyRigidSpinAroundY (engine/simulation.cpp:331-341)."""
    w = omega * T_UNIT
    body["velX"] = (w * body["posZ"].astype(np.float64)).astype(np.float32)
    body["velY"] = np.zeros_like(body["velY"])
    body["velZ"] = (-w * body["posX"].astype(np.float64)).astype(np.float32)


def _single_body_state(body):
    """makeCombinedFromSingleBody (engine/simulation.cpp:852-880)."""
    n = len(body["posX"])
    st = {k: body[k].copy() for k in BODY_FIELDS}
    st["h"] = body["h0"].copy()
    st["originalId"] = np.arange(n, dtype=np.uint32)
    return st


def _build_body(spec, n, body_id, grid, seed):
    """buildPlanet on the device, then (relaxSteps > 0) the engine's
    relaxation of the loaded single body (engine/simulation.cpp:1329-1357)."""
    p = engine.DeviceParticles(n)
    info = engine.build_planet(spec, n, p, offset=0, body_id=body_id, tracer_grid_res=grid, seed=seed)
    st = p.download()
    body = {k: st[k].copy() for k in BODY_FIELDS}
    radius_m = info["equatorialRadiusM"]
    if spec.relaxSteps > 0:
        _center_and_zero_bulk(body)
        for ax in ("velX", "velY", "velZ"):
            body[ax][:] = 0.0
        anchors = torch.from_numpy(body["tempK"].astype(np.float64)).cuda()
        sim = engine.Simulation(n)
        sim.load_state(_single_body_state(body))
        engine.relax_single_body(sim.p, sim.alt, sim.bvh, anchors, radius_m / L_UNIT, spec.relaxSteps)
        rel = sim.p.download()
        # copyRelaxedBodyToBuiltHost (engine/simulation.cpp:783-850): back to build order
        dst = np.where(rel["originalId"] < n, rel["originalId"], np.arange(n)).astype(np.int64)
        for k in ("posX", "posY", "posZ", "mass", "h0", "rho", "u", "tempK", "epsFail", "materialId",
                  "tracerIndex", "tracerIsOcean"):
            body[k][dst] = rel[k]
        for ax in ("velX", "velY", "velZ"):
            body[ax][:] = 0.0
        x, y, z = (rel[k].astype(np.float64) for k in ("posX", "posY", "posZ"))
        r = np.sqrt(x * x + y * y + z * z)
        tr = rel["tracerIndex"] >= 0
        body["tracerRestRadiusPsu"][dst[tr]] = r[tr].astype(np.float32)
        ok = tr & (r > 1.0e-9)
        for k, c in (("tracerRestNormalX", x), ("tracerRestNormalY", y), ("tracerRestNormalZ", z)):
            body[k][dst[ok]] = (c[ok] / r[ok]).astype(np.float32)
        if r.max() > 0.0:
            radius_m = float(r.max()) * L_UNIT
        _center_and_zero_bulk(body)
        _apply_spin(body, spec.spinOmegaRadS)
        del sim
    return body, radius_m, info


def load_scenario(cfg, sim=None):
    """Simulation::loadScenario on the device path.  Returns (Simulation,
    scenario dict with the bodies' radii, particle counts and orbit)."""
    t_spec, i_spec = cfg["target"], cfg["impactor"]
    total = cfg["total"]
    has_imp = i_spec.massKg > 0.0 and total >= 2
    tn, inum = total, 0
    if has_imp:
        mt = t_spec.massKg + i_spec.massKg
        k = int(math.floor(total * (i_spec.massKg / mt) + 0.5))
        k = min(max(k, min(total // 2, 16)), total - 1)
        inum, tn = k, total - k
    target, r_t, t_info = _build_body(t_spec, tn, 0, cfg["grid"], cfg["seed"])
    out = {"target_n": tn, "impactor_n": inum, "target_radius_psu": r_t / L_UNIT, "tracers": t_info["tracerCount"]}
    if has_imp:
        imp, r_i, _ = _build_body(i_spec, inum, 1, 0, cfg["seed"] + 1)
        mtp = float(np.sum(target["mass"].astype(np.float64)))
        mip = float(np.sum(imp["mass"].astype(np.float64)))
        mtot = mtp + mip
        rc = max(r_t / L_UNIT + r_i / L_UNIT, 1.0e-3)
        vesc = math.sqrt(2.0 * G_PSU * mtot / rc)
        vr = max(0.0, cfg["v_ratio"])
        vc = vr * vesc
        d0 = max(cfg["sep"], 1.0) * rc
        v0sq = vc * vc - 2.0 * G_PSU * mtot * (1.0 / rc - 1.0 / d0)
        if v0sq < 0.0:                               # engine/simulation.cpp:1407-1414
            rapo = rc / max(1.0 - vr * vr, 1.0e-6)
            d0 = min(max(0.98 * rapo, 1.01 * rc), d0)
            v0sq = max(0.0, vc * vc - 2.0 * G_PSU * mtot * (1.0 / rc - 1.0 / d0))
        v0 = math.sqrt(v0sq)
        b = min(max(cfg["b"], -1.2), 1.2)
        vperp = (rc * vc * b) / d0
        if abs(vperp) > 0.995 * v0:
            vperp = math.copysign(0.995 * v0, vperp)
        vrad = -math.sqrt(max(0.0, v0 * v0 - vperp * vperp))
        for body, f in ((target, -mip / mtot), (imp, mtp / mtot)):
            body["posX"] = (body["posX"].astype(np.float64) + f * d0).astype(np.float32)
            body["velX"] = (body["velX"].astype(np.float64) + f * vrad).astype(np.float32)
            body["velZ"] = (body["velZ"].astype(np.float64) + f * (-vperp)).astype(np.float32)
        # mergeTwoBodies (engine/simulation.cpp:882-947)
        st = {k: np.concatenate([target[k], imp[k]]) for k in BODY_FIELDS}
        st["h"] = st["h0"].copy()
        st["originalId"] = np.arange(tn + inum, dtype=np.uint32)
        _center_and_zero_bulk(st)
        out.update({"impactor_radius_psu": r_i / L_UNIT, "d0_psu": d0, "v_contact_psu": vc})
    else:
        st = _single_body_state(target)
    n = len(st["posX"])
    if sim is None:
        sim = engine.Simulation(n)
    sim.load_state(st)
    sim.evaluate_initial_forces()
    out["living_body_present"] = t_spec.archetype == 0
    return sim, out


def conservation_audit(step, particles, rt, living, steps, m_tot_kg, r_scale, v_esc):
    """The conservation figures of engine/headless_main.cpp:222-281: the
    device telemetry before and after `steps` calls of step() (each returns
    its dt in PSU), radiated energy integrated with the trapezoid rule, energy
    drift relative to |E0|, |dP| / (M v_esc) and |dL| / max(|L0|, 1e-6 M R
    v_esc).  particles() gives the device state to reduce (a DeviceParticles
    of this library or of any stepper that keeps the engine's SoA)."""
    def energy(t):
        return (t["kineticPsu"] + t["potentialPsu"] + t["internalPsu"]) * E_UNIT

    tel0 = engine.reduce_telemetry(particles(), rt, living)
    e0 = energy(tel0)
    p0 = np.array(tel0["momentumPsu"]) * M_UNIT * V_UNIT
    l0 = np.array(tel0["angularMomentumPsu"]) * L_ANG_UNIT
    prev_rad = tel0["radiatedPowerW"]
    e_rad = 0.0
    tel = tel0
    finite = math.isfinite(e0)
    for _ in range(steps):
        dt = step()
        tel = engine.reduce_telemetry(particles(), rt, living)
        curr = tel["radiatedPowerW"]
        e_rad += 0.5 * (prev_rad + curr) * dt * T_UNIT
        prev_rad = curr
        finite = finite and math.isfinite(energy(tel)) and math.isfinite(dt)
    drift = (energy(tel) + e_rad - e0) / max(abs(e0), 1.0)
    dp = np.array(tel["momentumPsu"]) * M_UNIT * V_UNIT - p0
    dl = np.array(tel["angularMomentumPsu"]) * L_ANG_UNIT - l0
    p_rel = float(np.linalg.norm(dp) / (m_tot_kg * v_esc)) if m_tot_kg * v_esc > 0 else 0.0
    l_ref = max(float(np.linalg.norm(l0)), m_tot_kg * r_scale * v_esc * 1.0e-6)
    l_rel = float(np.linalg.norm(dl) / l_ref)
    return {"energy_j_t0": e0, "energy_j_t1": energy(tel), "radiated_j": e_rad, "p0": p0, "l0": l0, "tel": tel,
            "energy_drift_rel": drift, "dp_rel": p_rel, "dl_rel": l_rel, "finite": finite}


def scenario_scales(cfg):
    """Total mass (kg), the length scale R_t + R_i (m) and v_esc over it, as
    the headless runner forms them for its thresholds."""
    r_t = engine.solve_hydrostatic(cfg["target"])[1]
    r_i = engine.solve_hydrostatic(cfg["impactor"])[1] if cfg["impactor"].massKg > 0.0 else 0.0
    m_tot_kg = cfg["target"].massKg + max(0.0, cfg["impactor"].massKg)
    r_scale = max(r_t + r_i, 1.0)
    return m_tot_kg, r_scale, math.sqrt(2.0 * G_SI * m_tot_kg / r_scale)


def run_headless(preset="LivingGaiaAsteroidCataclysm", particles=100000, steps=100, dt_max_sec=5.0,
                 relax_steps=None, verify=True):
    """engine/headless_main.cpp:162-281: load, step, conservation figures;
    returns a dict (ok = thresholds met when verify)."""
    cfg = preset_config(preset, particles, relax_steps)
    m_tot_kg, r_scale, v_esc = scenario_scales(cfg)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim, info = load_scenario(cfg)
    torch.cuda.synchronize()
    load_s = time.perf_counter() - t0
    rt, living = info["target_radius_psu"], info["living_body_present"]

    max_dt = float(max(1.0e-5, dt_max_sec) / T_UNIT)

    def step():
        torch.cuda.synchronize()
        ts = time.perf_counter()
        dt = sim.step(max_dt)
        step.seconds += time.perf_counter() - ts
        return dt
    step.seconds = 0.0
    a = conservation_audit(step, lambda: sim.p, rt, living, steps, m_tot_kg, r_scale, v_esc)
    step_s = step.seconds
    drift, p_rel, l_rel, finite = a["energy_drift_rel"], a["dp_rel"], a["dl_rel"], a["finite"]
    e0, e_rad, p0, l0, tel = a["energy_j_t0"], a["radiated_j"], a["p0"], a["l0"], a["tel"]

    def energy(t):
        return (t["kineticPsu"] + t["potentialPsu"] + t["internalPsu"]) * E_UNIT

    res = {"preset": preset, "particles": sim.p.count, "tracers": info["tracers"], "steps": steps,
           "energy_j_t0": e0, "energy_j_t1": energy(tel), "radiated_j": e_rad,
           "momentum_t0": p0.tolist(), "momentum_t1": (np.array(tel["momentumPsu"]) * M_UNIT * V_UNIT).tolist(),
           "angular_momentum_t0": l0.tolist(),
           "angular_momentum_t1": (np.array(tel["angularMomentumPsu"]) * L_ANG_UNIT).tolist(),
           "sim_time_sec": sim.sim_time * T_UNIT, "energy_drift_rel": drift, "dp_rel": p_rel, "dl_rel": l_rel,
           "max_temp_k": tel["maxTempK"], "max_pressure_gpa": tel["maxPressureGPa"], "finite": finite,
           "load_s": load_s, "step_s": step_s}
    res["ok"] = bool(finite and (not verify or (abs(drift) < 0.01 and p_rel < 1.0e-4 and l_rel < 0.005)))
    return res
