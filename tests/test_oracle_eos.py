"""The oracle's EOS against the reference's own EOS and its known answers.

Golden vectors come from engine/eos.cu compiled as host C++ (see
tests/golden/make_golden.py); the known-answer checks restate
tests/cpp/test_eos.cpp (analytic Tillotson pressures, HydrogenHelium
identities, phase branches, damaged tension).
"""
import math

import numpy as np
import pytest

import oracle

P_UNIT, RHO_UNIT, U_UNIT = 1.0e12, 1.0e6, 1.0e6
PAR = {
    0: dict(rho0=7800.0, a=0.5, b=1.5, A=1.28e11, B=1.05e11, E0=9.5e6, Eiv=2.4e6, Ecv=8.67e6, alpha=5.0, beta=5.0, cv=449.0, tRef=293.0, tMelt=1811.0),
    1: dict(rho0=2680.0, a=0.5, b=1.3, A=1.80e10, B=1.80e10, E0=1.6e7, Eiv=3.5e6, Ecv=1.8e7, alpha=5.0, beta=5.0, cv=790.0, tRef=293.0, tMelt=1600.0),
    2: dict(rho0=1000.0, a=0.7, b=0.15, A=2.18e9, B=1.325e10, E0=7.0e6, Eiv=4.19e5, Ecv=2.68e6, alpha=10.0, beta=5.0, cv=4184.0, tRef=273.15, tMelt=273.15),
    4: dict(rho0=2000.0, a=0.5, b=1.3, A=1.20e10, B=1.20e10, E0=1.6e7, Eiv=3.5e6, Ecv=1.8e7, alpha=5.0, beta=5.0, cv=800.0, tRef=293.0, tMelt=1500.0),
}
KH2, GAMMA, CV_HH = 2.08e5, 1.4, 8260.0


def eos1(mat, rho, u, d=0.0):
    P, cs, T, ph = oracle.eos_batch([mat], [rho], [u], [d])
    return float(P[0]), float(cs[0]), float(T[0]), int(ph[0])


def cold_si(mat, rho):
    p = PAR[mat]
    eta = rho / p["rho0"]
    if eta <= 1.0:
        return 0.0
    le = math.log(eta)
    return (p["A"] * (le + 1.0 / eta - 1.0) + p["B"] * (eta - 1.0 / eta - 2.0 * le)) / p["rho0"]


def pc_si(p, rho, ue):
    eta = rho / p["rho0"]
    mu = eta - 1.0
    return (p["a"] + p["b"] / (ue / (p["E0"] * eta * eta) + 1.0)) * rho * ue + p["A"] * mu + (p["B"] if mu >= 0 else 0.0) * mu * mu


def pe_si(p, rho, ue):
    eta = rho / p["rho0"]
    mu = eta - 1.0
    x = p["rho0"] / rho - 1.0
    den = ue / (p["E0"] * eta * eta) + 1.0
    return p["a"] * rho * ue + (p["b"] * rho * ue / den + p["A"] * mu * math.exp(-p["beta"] * x)) * math.exp(-p["alpha"] * x * x)


def test_oracle_eos_bit_exact_vs_reference_golden(golden_dir):
    g = np.load(golden_dir + "/eos_reference.npz")
    P, cs, T, ph = oracle.eos_batch(g["mat"], g["rho"], g["u"], g["dmg"])
    assert np.array_equal(P, g["P"])
    assert np.array_equal(cs, g["cs"])
    assert np.array_equal(T, g["T"])
    assert np.array_equal(ph, g["phase"])


def test_oracle_eos_vs_live_reference_library():
    ref = oracle.load_reference_eos()
    if ref is None:
        pytest.skip("reference checkout not present on this machine (golden vectors cover it)")
    rng = np.random.Generator(np.random.PCG64(11))
    n = 20000
    mat = rng.integers(0, 5, n).astype(np.uint8)
    rho = np.exp(rng.uniform(np.log(1e-7), np.log(0.05), n)).astype(np.float32)
    u = np.exp(rng.uniform(np.log(1e-4), np.log(200.0), n)).astype(np.float32)
    d = rng.uniform(0, 1, n).astype(np.float32)
    a = oracle.eos_batch(mat, rho, u, d)
    b = oracle.eos_batch(mat, rho, u, d, reference=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_cold_energy_analytic():   # tests/cpp/test_eos.cpp:164-195
    lib = oracle.load()
    for m in (0, 1, 2, 4):
        p = PAR[m]
        for eta in (0.5, 0.9, 1.0):
            assert lib.oracle_cold_energy(m, eta * p["rho0"] / RHO_UNIT) == 0.0
        prev = 0.0
        for eta in (1.05, 1.2, 1.5, 2.0, 3.0):
            rho = eta * p["rho0"]
            u = lib.oracle_cold_energy(m, rho / RHO_UNIT)
            exp = cold_si(m, rho) / U_UNIT
            assert u > prev
            assert abs(u - exp) <= 1e-10 * exp + 1e-12
            prev = u
    for rho in (0.178, 10.0, 100.0, 1000.0, 5000.0):
        u = lib.oracle_cold_energy(3, rho / RHO_UNIT)
        assert abs(u - KH2 * rho / U_UNIT) <= 1e-10 * KH2 * rho / U_UNIT + 1e-12


@pytest.mark.parametrize("mat", [0, 1, 2, 4])
def test_tillotson_regimes_and_damaged_tension(mat):   # tests/cpp/test_eos.cpp:197-275
    p = PAR[mat]
    rho0 = p["rho0"] / RHO_UNIT
    # compressed, eta = 1.5
    rho = np.float32(1.5 * rho0)
    rho_si = float(rho) * RHO_UNIT
    uc = oracle.load().oracle_cold_energy(mat, float(rho))
    ue_si = uc * U_UNIT + p["cv"] * 1000.0
    u = np.float32((uc * U_UNIT + p["cv"] * (p["tRef"] + 1000.0)) / U_UNIT)
    P, cs, T, _ = eos1(mat, rho, u)
    assert P > 0 and cs > 0 and T >= 3.0
    assert abs(P * P_UNIT - pc_si(p, rho_si, ue_si)) <= 1e-4 * abs(pc_si(p, rho_si, ue_si)) + 1e3
    Pd, _, _, _ = eos1(mat, rho, u, 1.0)
    assert Pd > 0 and abs(Pd - P) <= 1e-5 * abs(P) + 1e-12
    # two-phase, eta = 0.7
    rho = np.float32(0.7 * rho0)
    rho_si = float(rho) * RHO_UNIT
    ue = 0.5 * (p["Eiv"] + p["Ecv"])
    u = np.float32((p["cv"] * p["tRef"] + ue) / U_UNIT)
    P, cs, T, _ = eos1(mat, rho, u)
    exp = ((ue - p["Eiv"]) * pe_si(p, rho_si, ue) + (p["Ecv"] - ue) * pc_si(p, rho_si, ue)) / (p["Ecv"] - p["Eiv"])
    assert abs(P * P_UNIT - exp) <= 1e-4 * abs(exp) + 1e3
    # hot expanded, eta = 0.2
    rho = np.float32(0.2 * rho0)
    rho_si = float(rho) * RHO_UNIT
    ue = 2.0 * p["Ecv"]
    P, cs, T, _ = eos1(mat, rho, np.float32((p["cv"] * p["tRef"] + ue) / U_UNIT))
    assert P > 0 and abs(P * P_UNIT - pe_si(p, rho_si, ue)) <= 1e-4 * pe_si(p, rho_si, ue) + 1e3
    # damaged tension, eta = 0.9
    rho = np.float32(0.9 * rho0)
    u = np.float32(p["cv"] * p["tRef"] / U_UNIT)
    Pi = eos1(mat, rho, u, 0.0)[0]
    Pd = eos1(mat, rho, u, 1.0)[0]
    Ph = eos1(mat, rho, u, 0.5)[0]
    assert Pi < 0.0 and abs(Pd) <= 1e-12
    assert abs(Ph - 0.5 * Pi) <= 1e-5 * abs(Pi) + 1e-12


def test_hydrogen_helium_identities():   # tests/cpp/test_eos.cpp:277-316
    for rho_si, uth in ((0.178, 2.0e6), (50.0, 0.0), (200.0, 5.0e6), (1200.0, 2.5e7), (3500.0, 6.0e7)):
        u = np.float32((KH2 * rho_si + uth) / U_UNIT)
        P, cs, T, _ = eos1(3, np.float32(rho_si / RHO_UNIT), u)
        exp = KH2 * rho_si * rho_si + (GAMMA - 1.0) * rho_si * uth
        assert abs(P * P_UNIT - exp) <= 1e-4 * exp + 1.0
        c = max(0.05, math.sqrt(2.0 * KH2 * rho_si + GAMMA * (GAMMA - 1.0) * uth) / 1e3)
        assert abs(cs - c) <= 1e-4 * c + 1e-6


def test_phase_branches():   # tests/cpp/test_eos.cpp:342-409
    g = PAR[1]
    r0 = np.float32(g["rho0"] / RHO_UNIT)
    assert eos1(1, r0, np.float32(g["cv"] * 300 / U_UNIT))[3] == 0
    assert eos1(1, r0, np.float32(g["cv"] * 2200 / U_UNIT))[3] == 1
    assert eos1(1, r0, np.float32(g["cv"] * 15000 / U_UNIT))[3] == 3
    he = eos1(1, np.float32(0.5 * r0), np.float32((g["cv"] * g["tRef"] + 1.2 * g["Ecv"]) / U_UNIT))
    assert he[2] > 12000.0 and he[3] in (2, 3)
    w = PAR[2]
    w0 = np.float32(w["rho0"] / RHO_UNIT)
    assert eos1(2, w0, np.float32(w["cv"] * 200 / U_UNIT))[3] == 0
    assert eos1(2, w0, np.float32(w["cv"] * 300 / U_UNIT))[3] == 4
    assert eos1(2, np.float32(0.1 * w0), np.float32((w["cv"] * 1000 + w["Ecv"]) / U_UNIT))[3] == 2
    assert eos1(2, w0, np.float32(w["cv"] * 18000 / U_UNIT))[3] == 3
    rho = np.float32(100.0 / RHO_UNIT)
    uc = KH2 * 100.0 / U_UNIT
    assert eos1(3, rho, np.float32(uc + CV_HH * 500 / U_UNIT))[3] == 5
    assert eos1(3, rho, np.float32(uc + CV_HH * 12000 / U_UNIT))[3] == 3
