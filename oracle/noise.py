"""CPU restatement of the reference's detector noise, deepdrr/projector/analytic_generators.py:10-18,
given the Poisson variates. Test infrastructure only: the GPU tests feed it the variates the
library drew (drr_poisson_sample) and compare with drr_add_noise.

Per view, lambda = photon_prob * photon_count in float32 (numpy keeps float32 for a float32 array
times a Python int), then in float64:
    shot = (k - lambda) * intensity / lambda
    out  = clip(intensity + convolve2d(shot, K, mode="same"), 0, 10e30)
The electronic-noise term is scaled by 0 in the reference (analytic_generators.py:7) and omitted.
"""
from __future__ import annotations

import numpy as np
from scipy.signal import convolve2d

# analytic_generators.py:6 (Wang et al., Med Phys 41(7), 2014)
KERNEL_SHOT = np.array([[0.03, 0.06, 0.02], [0.11, 0.98, 0.11], [0.02, 0.06, 0.03]])


def add_noise_given_counts(intensity: np.ndarray, photon_prob: np.ndarray, counts: np.ndarray,
                           photon_count: float) -> np.ndarray:
    """[N, H, W] float64 noisy images from the same variates `counts` [N, H, W]."""
    lam = photon_prob.astype(np.float32) * np.float32(photon_count)
    out = np.empty(intensity.shape, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in range(intensity.shape[0]):
            shot = (counts[i].astype(np.float64) - lam[i].astype(np.float64)) * intensity[i].astype(np.float64) \
                / lam[i].astype(np.float64)
            shot = convolve2d(shot, KERNEL_SHOT, mode="same")
            out[i] = np.clip(intensity[i] + shot, 0.0, 10e30)
    return out
