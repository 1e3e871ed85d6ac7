"""Host side of the batched DMC driver for one crowd.

The device runs every DMC step (fixed-node sweep, local energy, branch weights) and
the walker copies of population control (qmcg_dmc_step, qmcg_dmc_reconfigure).  The
host keeps what the reference keeps on the host: the branching parameters of
SFNBranch (trial and reference energies, effective time step, branch cutoffs;
src/QMCDrivers/SFNBranch.cpp:94-232, 285-320) and the per-step ensemble record of
DMCBatched::run (src/QMCDrivers/DMC/DMCBatched.cpp:442-520).  Population control
keeps the crowd's walker count (the comb of WalkerReconfiguration); the population
weight before the comb feeds E_trial as SFNBranch::updateParamAfterPopControl does.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .crowd import Crowd


@dataclasses.dataclass
class BranchEngine:
    """The parameters SFNBranch carries between DMC steps (its vParam subset)."""

    tau: float
    num_electrons: int
    target_walkers: int
    feedback: float = 1.0
    sigma_bound: float = 10.0
    warmup_steps: int = 10
    e_trial: float = 0.0
    e_ref: float = 0.0
    e_now: float = 0.0
    tau_eff: float = 0.0
    sigma2: float = 0.0
    branch_cutoff: float = 0.0
    branch_max: float = 0.0
    r2_accepted: float = 0.0
    r2_proposed: float = 0.0
    warmup_left: int = 0
    ref_weight: float = 0.0
    ref_energy_sum: float = 0.0

    def set_branch_cutoff(self, variance: float, target_sigma: float, max_sigma: float):
        """The default ("classic") cutoff scheme of SFNBranch::setBranchCutoff."""
        self.branch_cutoff = min(max(variance * target_sigma, max_sigma), 2.5 / self.tau)
        self.branch_max = 1.5 * self.branch_cutoff

    def start(self, energies):
        """SFNBranch::initParam from the walkers' local energies."""
        e = np.asarray(energies, np.float64)
        self.e_trial = self.e_ref = self.e_now = float(e.mean())
        self.sigma2 = float(e.var())
        self.tau_eff = self.tau
        self.warmup_left = self.warmup_steps
        self.set_branch_cutoff(self.sigma2, self.sigma_bound, 50.0)

    def params(self) -> dict:
        return {"e_trial": self.e_trial, "e_ref": self.e_ref, "tau_eff": self.tau_eff,
                "branch_cutoff": self.branch_cutoff, "branch_max": self.branch_max}

    def update(self, sums):
        """SFNBranch::updateParamAfterPopControl with population control on, from the
        ensemble sums of a step (sum w, sum w E, sum w E^2, sum r2 accepted, sum r2 proposed)."""
        wsum, ewsum, e2wsum, r2a, r2p = (float(x) for x in sums)
        self.e_now = ewsum / wsum
        variance = e2wsum / wsum - self.e_now * self.e_now
        self.r2_accepted += r2a
        self.r2_proposed += r2p
        if self.r2_proposed > 0:
            self.tau_eff = self.tau * self.r2_accepted / self.r2_proposed
        log_n = math.log(self.target_walkers)
        if self.warmup_left > 0:
            self.e_ref = self.e_now
            self.e_trial = self.e_now + (log_n - math.log(wsum)) / self.tau
            self.warmup_left -= 1
            if self.warmup_left == 0:
                self.sigma2 = variance
                self.set_branch_cutoff(self.sigma2, self.sigma_bound, 10.0)
        else:
            # the reference energy is the weighted average of the step energies since warm-up
            self.ref_weight += wsum
            self.ref_energy_sum += wsum * self.e_now
            self.e_ref = self.ref_energy_sum / self.ref_weight
            self.e_trial = self.e_ref + self.feedback * (log_n - math.log(wsum))


class DMCDriver:
    """DMC steps of one crowd: device step, population control, branching parameters."""

    def __init__(self, crowd: Crowd, tau: float, seed: int, warmup_steps: int = 10, feedback: float = 1.0,
                 flush: int = 0, recompute_every: int = 0):
        self.crowd, self.tau, self.seed = crowd, tau, seed
        self.flush, self.recompute_every = flush, recompute_every
        self.rng = np.random.default_rng(seed)
        self.engine = BranchEngine(tau=tau, num_electrons=crowd.ne, target_walkers=crowd.nw, feedback=feedback,
                                   warmup_steps=warmup_steps)
        self.engine.start(crowd.dmc_init())
        self.history = []

    def step(self) -> dict:
        out = self.crowd.dmc_step(self.tau, self.seed, recompute_every=self.recompute_every, flush=self.flush,
                                  **self.engine.params())
        src = self.crowd.dmc_reconfigure(self.rng.random())
        rec = {"e_now": float(out["sums"][1] / out["sums"][0]), "weight": float(out["sums"][0]),
               "e_trial": self.engine.e_trial, "e_ref": self.engine.e_ref, "tau_eff": self.engine.tau_eff,
               "copied": int(np.sum(src != np.arange(src.size))), "accepted": out["accepted"],
               "rejected": out["rejected"]}
        self.engine.update(out["sums"])
        self.history.append(rec)
        return rec

    def run(self, nsteps: int):
        return [self.step() for _ in range(nsteps)]
