"""Synthetic input decks for the benchmark shapes (no dataset is involved).

Each deck gives the grid, one electron plasma species and Gaussian electron beams in the
reference's JSON-key vocabulary (simulation.grid/box/max_mode/iter_*, species ppc and
num_theta, beam gauss_center/gauss_sigma/total_charge/total_num/gamma/uth).  Plasma
"a x b particles per cell" is loaded as ppc = (a, b // 8) with num_theta = 8.  Beam
charge is set from the peak density n_b as Q = n_b (2 pi)^(3/2) sigma_r^2 sigma_xi, and
uth_perp = eps_n / sigma_r.  Beam centres sit 3 sigma_xi behind the box head; ranges are
+-5 sigma (clipped to the box by the loader).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field


@dataclass
class BeamSpec:
    n_b: float
    sigma_r: float
    sigma_xi: float
    center_xi: float
    num: int
    gamma: float = 20000.0
    eps_n: float = 1.0e-3
    x0: float = 0.0
    qm: float = -1.0

    @property
    def charge(self) -> float:
        return self.n_b * (2.0 * math.pi) ** 1.5 * self.sigma_r ** 2 * self.sigma_xi

    def load_args(self, nz, dxi):
        box = nz * dxi
        c = (self.x0, 0.0, self.center_xi)
        s = (self.sigma_r, self.sigma_r, self.sigma_xi)
        lo = (self.x0 - 5 * self.sigma_r, -5 * self.sigma_r, max(0.0, self.center_xi - 5 * self.sigma_xi))
        hi = (self.x0 + 5 * self.sigma_r, 5 * self.sigma_r, min(box, self.center_xi + 5 * self.sigma_xi))
        uth = (self.eps_n / self.sigma_r, self.eps_n / self.sigma_r, 0.0)
        return dict(tot_num=self.num, tot_charge=self.charge, qm=self.qm, gamma=self.gamma, center=c, sigma=s,
                    range_lo=lo, range_hi=hi, uth=uth)


@dataclass
class Deck:
    name: str
    nr: int
    nz: int
    max_mode: int
    dr: float
    dxi: float
    ppc: tuple
    num_theta: int
    uth: float
    seed: int
    beams: list = field(default_factory=list)
    iter_max: int = 50
    iter_reltol: float = 1.0e-6
    iter_abstol: float = 0.0
    dt: float = 10.0
    n_steps: int = 1
    smooth_order: int = 0

    @property
    def np_per_slice(self) -> int:
        return self.nr * self.ppc[0] * self.ppc[1] * self.num_theta

    def scaled(self, nz=None, beam_frac=None, **kw) -> "Deck":
        """A copy with fewer slices / beam particles (for parity tests and CPU samples)."""
        import copy
        d = copy.deepcopy(self)
        if nz is not None:
            d.nz = nz
        if beam_frac is not None:
            for b in d.beams:
                b.num = max(1, int(b.num * beam_frac))
        for k, v in kw.items():
            setattr(d, k, v)
        return d


def c1() -> Deck:
    """Plain FP64 small blowout: M=1, nr=256, dr=0.04, 256 slices, 4x8 ppc, cold plasma."""
    return Deck("c1_blowout_m1_nr256", 256, 256, 1, 0.04, 0.04, (4, 1), 8, 0.0, 0,
                beams=[BeamSpec(3.0, 0.5, 1.0, 3.0, 1_000_000)])


def c2() -> Deck:
    """Hosing blowout: M=2, nr=512, dr=0.02, 1024 slices, 8x16 ppc, thermal plasma, driver + witness."""
    return Deck("c2_hosing_m2_nr512", 512, 1024, 2, 0.02, 0.02, (8, 2), 8, 1.0e-3, 1,
                beams=[BeamSpec(5.0, 0.3, 0.8, 2.4, 4_000_000, x0=0.03),
                       BeamSpec(10.0, 0.2, 0.3, 6.4, 2_000_000)])


def c5() -> Deck:
    """Production shape: M=4, nr=2048, dr=0.01, 4096 slices, 16x32 ppc (1.05e6 particles per slice)."""
    return Deck("c5_production_m4_nr2048", 2048, 4096, 4, 0.01, 0.01, (16, 4), 8, 0.0, 4,
                beams=[BeamSpec(10.0, 0.2, 0.5, 1.5, 50_000_000, gamma=40000.0),
                       BeamSpec(20.0, 0.1, 0.3, 5.5, 50_000_000, gamma=40000.0)], n_steps=10)


def c3(n: int = 64, seed: int = 2) -> list:
    """Batched scan: n independent simulations of uneven size (seed 2).  nr uniform in
    {128, 256, 512, 1024} with dr = 10.24 / nr, max mode uniform in 0..4, particles per cell
    a x b with a uniform in 4..8 and b in {8, 16}, driver peak density log-uniform in
    [0.5, 20], sigma_r uniform in [0.2, 1.0], sigma_xi = 1, 512 slices of dxi = 0.04, the
    driver centre 3 sigma_xi behind the box head, 200,000 beam particles per simulation."""
    import random
    rng = random.Random(seed)
    out = []
    for k in range(n):
        nr = rng.choice([128, 256, 512, 1024])
        M = rng.randint(0, 4)
        a, b = rng.randint(4, 8), rng.choice([8, 16])
        n_b = math.exp(rng.uniform(math.log(0.5), math.log(20.0)))
        sig_r = rng.uniform(0.2, 1.0)
        out.append(Deck(f"c3_{k:02d}_m{M}_nr{nr}", nr, 512, M, 10.24 / nr, 0.04, (a, b // 8), 8, 0.0,
                        seed * 1000 + k, beams=[BeamSpec(n_b, sig_r, 1.0, 3.0, 200_000)]))
    return out


DECKS = {"c1": c1, "c2": c2, "c5": c5}
