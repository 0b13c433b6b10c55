"""The engine's per-frame telemetry snapshot from the device reduction.

astraea_gb300_reduce_telemetry (engine.reduce_telemetry) returns the sums,
extremes and remnant classification of the O(N) loops of
computeTelemetryFromDevice (engine/simulation.cpp:948-1285) in PSU.  The
scalar code that follows those loops in the engine -- unit conversion,
energy drift, virial ratio, living-body COM / radius / spin, impactor COM,
mass fractions and the collision-outcome rules (:1057-1285) -- runs here on
the host, with the engine's constants, and yields the engine's
TelemetrySnapshot fields (engine/types.hpp:81-111) under the same names.
"""
import math

# PSU units (engine/units.hpp:14-27)
L_UNIT_M = 1.0e6
M_UNIT_KG = 1.0e24
T_UNIT_S = 1.0e3
V_UNIT_MS = L_UNIT_M / T_UNIT_S
E_UNIT_J = M_UNIT_KG * V_UNIT_MS * V_UNIT_MS
L_ANG_UNIT = M_UNIT_KG * L_UNIT_M * V_UNIT_MS
G_PSU = 6.67430e-11 * M_UNIT_KG * T_UNIT_S * T_UNIT_S / (L_UNIT_M * L_UNIT_M * L_UNIT_M)

# CollisionOutcome (engine/types.hpp) in declaration order
APPROACHING, MERGING, GRAZE_AND_MERGE, HIT_AND_RUN, CATASTROPHIC_DISRUPTION = range(5)


def telemetry_snapshot(t, ctx):
    """TelemetrySnapshot fields from the device reduction `t` (a dict of
    AstraeaTelemetry fields) and the engine state `ctx`: targetRadiusPsu,
    impactorRadiusPsu, livingBodyPresent, hasImpacted, qRatioQrd,
    impactParamB, impactVelocityRatioVesc, targetSpinOmegaRadS, frameSeq,
    simTimeSec, radiatedEnergyJ, initialTotalEnergyJ.  Returns (snapshot,
    hasImpacted after this frame, initialTotalEnergyJ after this frame) --
    the two pieces of engine state the snapshot updates."""
    s = {}
    ke, pe, ie = (t["kineticPsu"] * E_UNIT_J, t["potentialPsu"] * E_UNIT_J, t["internalPsu"] * E_UNIT_J)
    s["kineticEnergyJ"], s["potentialEnergyJ"], s["internalEnergyJ"] = ke, pe, ie
    s["totalEnergyJ"] = ke + pe + ie
    e0 = ctx["initialTotalEnergyJ"]
    if ctx["frameSeq"] == 0 and ctx["simTimeSec"] == 0.0:
        e0 = s["totalEnergyJ"]
        s["energyDriftRel"] = 0.0
    else:
        s["energyDriftRel"] = (s["totalEnergyJ"] + ctx["radiatedEnergyJ"] - e0) / max(abs(e0), 1.0)
    s["initialTotalEnergyJ"] = e0
    mom = M_UNIT_KG * V_UNIT_MS
    for k, ax in enumerate("XYZ"):
        s["momentum" + ax] = t["momentumPsu"][k] * mom
        s["angularMomentum" + ax] = t["angularMomentumPsu"][k] * L_ANG_UNIT
    s["virialRatio"] = (-2.0 * ke / pe) if abs(pe) > 1.0 else 0.0
    s["maxTempK"], s["maxPressureGPa"] = t["maxTempK"], t["maxPressureGPa"]
    sys_com, liv = t["sysComPsu"], t["livingComPsu"]
    rt = ctx["targetRadiusPsu"]
    for k, ax in enumerate("XYZ"):
        s["livingBodyComKm" + ax] = 0.0
        s["impactorComKm" + ax] = 0.0
    s["livingBodyRadiusKm"] = s["livingBodySpinRadS"] = 0.0
    if ctx["livingBodyPresent"]:
        for k, ax in enumerate("XYZ"):
            s["livingBodyComKm" + ax] = (liv[k] - sys_com[k]) * 1000.0
        s["livingBodyRadiusKm"] = rt * 1000.0
        s["livingBodySpinRadS"] = ((t["spinLPsu"] / t["spinIPsu"]) / T_UNIT_S if t["spinIPsu"] > 0.0
                                   else ctx["targetSpinOmegaRadS"])
    m0, m1 = t["massBody0Psu"], t["massOtherPsu"]
    if m1 > 0.0:
        for k, ax in enumerate("XYZ"):
            s["impactorComKm" + ax] = (t["comOtherPsu"][k] - sys_com[k]) * 1000.0
    mt = t["totalMassPsu"]
    if mt > 0.0:
        s["boundMassFrac"] = t["boundPlanetMassPsu"] / mt
        s["diskMassFrac"] = t["diskMassPsu"] / mt
        s["ejectaMassFrac"] = t["ejectaMassPsu"] / mt
    else:
        s["boundMassFrac"], s["diskMassFrac"], s["ejectaMassFrac"] = 1.0, 0.0, 0.0
    impacted = bool(ctx["hasImpacted"])
    if m1 <= 0.0:
        s["outcome"] = MERGING
    else:
        c0, c1 = t["comBody0Psu"], t["comOtherPsu"]
        v0, v1 = t["velBody0Psu"], t["velOtherPsu"]
        r = [c1[k] - c0[k] for k in range(3)]
        rv = [v1[k] - v0[k] for k in range(3)]
        d_sep = math.sqrt(sum(x * x for x in r))
        r_dot_v = sum(r[k] * rv[k] for k in range(3))
        contact = rt + ctx["impactorRadiusPsu"]
        if d_sep <= 1.05 * contact or t["maxDamage"] > 0.25 or r_dot_v >= 0.0:
            impacted = True
        if not impacted and d_sep > 1.05 * contact and r_dot_v < 0.0:
            s["outcome"] = APPROACHING
        else:
            bound_frac = t["impactorBoundMassPsu"] / m1
            b_abs = abs(ctx["impactParamB"])
            two_body = 0.5 * sum(x * x for x in rv) - G_PSU * (m0 + m1) / max(d_sep, 1.0e-3)
            q = ctx["qRatioQrd"]
            if s["boundMassFrac"] < 0.50 or (q >= 1.0 and (s["ejectaMassFrac"] >= 0.15 or s["boundMassFrac"] < 0.72)):
                s["outcome"] = CATASTROPHIC_DISRUPTION
            elif r_dot_v > 0.0 and d_sep > 1.05 * contact and (bound_frac < 0.50 or two_body > 0.0):
                s["outcome"] = HIT_AND_RUN
            elif b_abs >= 0.50 and ctx["impactVelocityRatioVesc"] > 1.25 and bound_frac < 0.45:
                s["outcome"] = HIT_AND_RUN
            elif b_abs >= 0.45:
                s["outcome"] = GRAZE_AND_MERGE
            else:
                s["outcome"] = MERGING
    return s, impacted, e0
