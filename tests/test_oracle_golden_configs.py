"""Pins the CPU oracle against the reference's own propagation at the
benchmark configurations (fixtures made by tests/golden/make_golden.py, cases
ocs_c1, asym_j10, c1_j10):

* ocs_c1_j20: linear OCS J <= 20 with all M (dim 441), z pulse 5e11 W/cm^2,
  FWHM 300 fs at 1 ps, 0-3 ps at 10 fs (300 steps): <cos^2>, <cos> and
  J-populations every step, states every 10 steps;
* asym_j10: D2 asymmetric top J <= 10 (dim 1,771), DC 20 kV/cm + 1e12 W/cm^2
  pulse at 35 deg, 50 steps of 5 fs through the pulse maximum, T = 5 K
  ensemble of 22 vectors (two of them here: the oracle is a scalar loop);
* c1_j10: a C1 molecule J <= 10, 10 steps under a tilted pulse.

CPU only. Tolerances: states 1e-10 relative, observables 1e-9 absolute.
"""
import os

import numpy as np

from oracle import fixtures
from oracle.cartens import add_cartens, split
from oracle.tdse import OTDSE

from conftest import GOLDEN

STATE_RTOL = 1e-10
OBS_ATOL = 1e-9


def _load(name):
    return fixtures.load(os.path.join(GOLDEN, name))


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _pops(T, v):
    d = split(T, v, "1")
    return np.array([sum(float(np.sum(np.abs(d[J][s]) ** 2)) for s in T.symlist1[J]) for J in T.Jlist1])


def test_ocs_c1_configuration_matches_reference():
    d, meta = _load("ocs_c1_j20.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    Hac = fixtures.tensor(d, meta, "pol") * meta["scale"]
    c2 = fixtures.tensor(d, meta, "cos2").tomat(form="full", cart="0")
    c1 = fixtures.tensor(d, meta, "cos").tomat(form="full", cart="0")
    p = meta["tdse"]
    td = OTDSE(t_start=p["t_start"], t_end=p["t_end"], dt=p["dt"])
    tc = td.time_grid()
    assert len(tc) == 300 and np.abs(np.asarray(tc) - d["tc"]).max() < 1e-12
    v = td.init_state(h0, temp=0)
    assert np.array_equal(v, d["vec0"])
    saved = {int(s): k for k, s in enumerate(d["state_steps"])}
    for i in range(len(tc)):
        Hac.field(d["fields"][i])
        v, t2 = td.update(Hac, v, H0=h0)
        assert abs(t2 - d["times"][i]) < 1e-12
        assert abs(np.vdot(v[0], c2.dot(v[0])).real + 1 / 3 - d["cos2"][i]) < OBS_ATOL
        assert abs(np.vdot(v[0], c1.dot(v[0])).real - d["cos"][i]) < OBS_ATOL
        assert np.abs(_pops(h0, v[0]) - d["pops"][i]).max() < OBS_ATOL
        if i in saved:
            assert _rel(v[0], d["states"][saved[i]]) < STATE_RTOL, i


def test_asym_j10_two_vectors_match_reference():
    d, meta = _load("asym_j10.npz")
    sc = meta["scales"]
    h0 = fixtures.tensor(d, meta, "h0")
    Hdc = (fixtures.tensor(d, meta, "dip") * meta["dc"]) * sc["dc"]
    Hac = fixtures.tensor(d, meta, "pol") * sc["ac"]
    c2 = fixtures.tensor(d, meta, "cos2").tomat(form="full", cart="0")
    c1 = fixtures.tensor(d, meta, "cos").tomat(form="full", cart="0")
    p = meta["tdse"]
    td = OTDSE(t_start=p["t_start"], t_end=p["t_end"], dt=p["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    assert v0.shape == d["vec0"].shape and np.abs(v0 - d["vec0"]).max() < 1e-14
    v = v0[:2].copy()
    saved = {int(s): k for k, s in enumerate(d["state_steps"])}
    for i in range(len(tc)):
        Hac.field(d["fields"][i])
        v, _ = td.update(add_cartens(Hdc, Hac), v, H0=h0)
        for r in range(2):
            assert abs(np.vdot(v[r], c2.dot(v[r])).real - d["cos2"][i, r]) < OBS_ATOL
            assert abs(np.vdot(v[r], c1.dot(v[r])).real - d["cos"][i, r]) < OBS_ATOL
            assert np.abs(_pops(h0, v[r]) - d["pops"][i, r]).max() < OBS_ATOL
        if i in saved:
            assert _rel(v, d["states"][saved[i]]) < STATE_RTOL, i
    assert _rel(v, d["final"][:2]) < STATE_RTOL


def test_c1_molecule_short_run_matches_reference():
    d, meta = _load("c1_j10.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    Hac = fixtures.tensor(d, meta, "pol") * meta["scale"]
    c2 = fixtures.tensor(d, meta, "cos2").tomat(form="full", cart="0")
    p = meta["tdse"]
    td = OTDSE(t_start=p["t_start"], t_end=p["t_end"], dt=p["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=2, thresh=1e-2)
    assert v0.shape == d["vec0"].shape and np.abs(v0 - d["vec0"]).max() < 1e-14
    v = v0[:4].copy()
    for i in range(len(tc)):
        Hac.field(d["fields"][i])
        v, _ = td.update(Hac, v, H0=h0)
        for r in range(4):
            assert abs(np.vdot(v[r], c2.dot(v[r])).real - d["cos2"][i, r]) < OBS_ATOL
    assert _rel(v, d["final"]) < STATE_RTOL
