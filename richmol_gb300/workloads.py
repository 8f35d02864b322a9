"""Synthetic workloads of the propagation benchmark (molecules, fields, grids).

No public dataset is involved: the inputs are fixed synthetic molecules and
pulses, built with the in-house factor builder (richmol_gb300.rot).

* ``linear_ocs``  linear O-C-S (C-O 1.16 A, C-S 1.56 A), mu_z = 0.28 au,
  alpha = diag(35, 35, 80) au, J = 0..Jmax (default 20) with all M; z pulse
  5e11 W/cm^2, FWHM 300 fs at 1 ps, cycle averaged; 0-3 ps, dt = 10 fs.
* ``asym_top``    asymmetric top (Bx, By, Bz) = (A, B, C) = (9.0, 5.0, 3.2) cm^-1,
  Watson A with Delta_J = Delta_JK = Delta_K = 1e-3 cm^-1, D2, mu = (0, 0, -0.73)
  au, alpha = diag(9.1, 9.9, 9.4) au, J = 0..Jmax (default 40) with all M and k;
  DC field 20 kV/cm along z plus a 1e12 W/cm^2 FWHM 500 fs pulse polarised at
  35 deg to the DC field, centred at 1 ps; dt = 5 fs, 4000 steps.
"""
import numpy as np

from . import rot
from .convert_units import AUdip_x_Vm_to_invcm, AUpol_x_Vm_to_invcm


class Workload:
    """Operators, field schedule and time grid of one propagation problem."""

    def __init__(self, name, mol, Jmax, t_start, t_end, dt, dc, pulse, temp=0):
        self.name = name
        self.mol = mol
        self.Jmax = Jmax
        self.t_start, self.t_end, self.dt = t_start, t_end, dt
        self.dc = None if dc is None else np.asarray(dc, dtype=np.float64)
        self.pulse = pulse  # (t0, fwhm, intensity, direction)
        self.temp = temp
        self.sol = rot.Solution(mol, Jmax=Jmax)
        self.h0 = rot.lab_tensor("h0", self.sol)
        self.pol = rot.lab_tensor(mol.pol, self.sol)
        self.dip = rot.lab_tensor(mol.dip, self.sol) if mol.dip is not None and np.any(mol.dip) else None
        self.cos2 = rot.lab_tensor("cos2theta", self.sol)
        self.cos = rot.lab_tensor("costheta", self.sol)
        self.Hac = self.pol * (-0.5 * AUpol_x_Vm_to_invcm())
        self.Hdc = None
        if self.dc is not None and self.dip is not None:
            self.Hdc = (self.dip * list(self.dc)) * (-1 * AUdip_x_Vm_to_invcm())
        self.dim = sum(self.h0.dim1[J][s] for J in self.h0.Jlist1 for s in self.h0.symlist1[J])

    def field(self, t):
        t0, fwhm, inten, direction = self.pulse
        return rot.pulse_field(t, t0, fwhm, inten, direction)

    def hamiltonian(self, t):
        """H(t) without H0: the DC term plus the pulse term at time t."""
        self.Hac.field(self.field(t))
        return self.Hac if self.Hdc is None else self.Hdc + self.Hac

    @property
    def nsteps(self):
        return int((self.t_end - self.t_start) / self.dt)


def linear_ocs(Jmax=20):
    mol = rot.Molecule(xyz=[("C", 0, 0, 0), ("O", 0, 0, -1.16), ("S", 0, 0, 1.56)],
                       dip=[0, 0, 0.28], pol=np.diag([35.0, 35.0, 80.0]))
    return Workload("linear_ocs_J%d" % Jmax, mol, Jmax, 0.0, 3.0, 0.01, None,
                    (1.0, 0.3, 5e11, [0, 0, 1]))


def asym_top(Jmax=40, dt=0.005, nsteps=4000):
    mol = rot.Molecule(B=(9.0, 5.0, 3.2), sym="D2", watson=dict(DeltaJ=1e-3, DeltaJK=1e-3, DeltaK=1e-3),
                       dip=[0, 0, -0.73], pol=np.diag([9.1, 9.9, 9.4]))
    beta = np.deg2rad(35.0)
    return Workload("asym_top_D2_J%d" % Jmax, mol, Jmax, 0.0, nsteps * dt, dt, [0.0, 0.0, 20e3 * 1e2],
                    (1.0, 0.5, 1e12, [np.sin(beta), 0.0, np.cos(beta)]))


class Ensemble:
    """Thermal ensemble of a workload: eigenstates of H0 (unit vectors in its
    eigenbasis) in energy order, the Boltzmann weight of each at T, padded with
    the next-lowest states to nvec right-hand sides."""

    def __init__(self, wl, nvec, temp, wmin=1e-5):
        import scipy.constants as const
        wl.h0.field([0, 0, 1])
        enr = wl.h0.tomat(form="full").diagonal().real
        order = np.argsort(enr, kind="stable")
        w = np.exp(-(enr[order] - enr[order[0]]) * (const.h * const.c * 100.0) / (const.k * temp))
        w /= w.sum()
        self.n_natural = int(np.sum(w >= wmin))
        self.nvec = int(nvec)
        self.index = order[: self.nvec]
        self.weights = w[: self.nvec]

    def vectors(self, dim):
        v = np.zeros((self.nvec, dim), np.complex128)
        v[np.arange(self.nvec), self.index] = 1.0
        return v


def thermal_asym_top(Jmax=30, nvec=4096, temp=5.0, dt=0.01, nsteps=3000):
    """Batched configuration: the asymmetric top of ``asym_top`` with J = 0..30,
    its T = 5 K ensemble (states with Boltzmann weight >= 1e-5, padded to 4096
    vectors), same DC field and pulse, 3000 steps of 10 fs."""
    wl = asym_top(Jmax=Jmax, dt=dt, nsteps=nsteps)
    wl.name = "thermal_asym_top_D2_J%d_%dvec" % (Jmax, nvec)
    return wl, Ensemble(wl, nvec, temp)


def uneven_molecules(n, seed=0, jmax_range=(10, 50), t_end=20.0, dt=0.01):
    """The uneven-size batch: n asymmetric tops without symmetry (C1), each
    drawn as a propagation request is (richmol_gb300.serve.draw_request: A >= B
    >= C log-uniform in 0.05-5 cm^-1, Jmax uniform in ``jmax_range``, random
    polarizability, its own pulse centred at t_end / 2), 0 - t_end ps at dt."""
    from .serve import draw_request
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        r = draw_request(rng, i, 0.0, jmax_range=jmax_range, t_end=t_end, dt=dt)
        mol = rot.Molecule(B=r.abc, sym="C1", pol=r.pol)
        out.append(Workload("molecule_%d_J%d" % (i, r.jmax), mol, r.jmax, 0.0, t_end, dt, None, r.pulse))
    return out


def ground_state(wl):
    """Unit vector of the lowest eigenstate of the workload's H0."""
    wl.h0.field([0, 0, 1])
    e = wl.h0.tomat(form="full").diagonal().real
    v = np.zeros(wl.dim, np.complex128)
    v[int(np.argmin(e))] = 1.0
    return v
