"""CPU restatement of the DMC branch step (test infrastructure only: tests/ use it as
the checker of the device branch weights and of the library's population control).

  branch_weight   SFNBranch::branchWeight, src/QMCDrivers/SFNBranch.h:199-208
  comb            WalkerReconfiguration::getIndexPermutation,
                  src/QMCDrivers/DMC/WalkerReconfiguration.cpp:30-107
"""
from __future__ import annotations

import numpy as np


def branch_weight(enew, eold, e_trial, e_ref, tau_eff, branch_cutoff, branch_max):
    """exp(t (2 E_trial - E_new - E_old)), t = tau_eff / 2 filtered by the energy window
    x = max(E_ref - E_new, E_ref - E_old): scaled by 1 - (x - cutoff) / (max - cutoff)
    above the cutoff, zero above max."""
    enew = np.asarray(enew, np.float64)
    eold = np.asarray(eold, np.float64)
    t = np.full(enew.shape, 0.5 * tau_eff)
    x = np.maximum(e_ref - enew, e_ref - eold)
    filt = 1.0 / (branch_max - branch_cutoff)
    t = np.where(x > branch_max, 0.0, np.where(x > branch_cutoff, t * (1.0 - (x - branch_cutoff) * filt), t))
    return np.exp(t * (e_trial * 2.0 - enew - eold))


def comb(weights, u: float):
    """Sources of every slot after population control with a fixed walker count, and the
    number of walkers kept, as a scalar loop over the cumulative weights."""
    w = np.abs(np.asarray(weights, np.float64))
    nw = w.size
    wtot = 0.0
    for x in w:
        wtot += x
    nw_inv = 1.0 / nw
    dstep = u * nw_inv
    zeta = [wtot * (dstep + i * nw_inv) for i in range(nw)] + [wtot + 1.0]
    ind, wcur = 0, 0.0
    copies = []
    for iw in range(nw):
        tryp = wcur + w[iw]
        ni = 0
        while zeta[ind] < tryp and zeta[ind] >= wcur:
            ind += 1
            ni += 1
        wcur += w[iw]
        copies.append(ni)
    plus, minus = [], []
    for iw, m in enumerate(copies):
        if m > 1:
            plus += [iw] * (m - 1)
        elif m == 0:
            minus.append(iw)
    src = np.arange(nw, dtype=np.int32)
    for im, ip in zip(minus, plus):
        src[im] = ip
    return src, int(sum(1 for m in copies if m > 0))
