"""The benchmark's single-step workload built without the engine -- TEST
INFRASTRUCTURE ONLY.

The CPU baseline and the reference arm of bench.py time the oracle on the
1536-channel x 2048-DM x 24576-sample 8-bit workload.  This module builds
that workload from numpy and the oracle alone, so that the CPU timing runs in
a process that never loads the engine's library.  It draws the same bytes as
the engine's seeded generator (dedispersion_gb300/synthetic.py:
make_observation, zapped_mask, make_input with injected pulses), which
tests/test_oracle_workload.py checks byte for byte:

* observation: 1536 channels of 0.1953125 MHz from 1220 MHz, 81.92 us
  sampling, 24576 samples, 2048 DMs from 0 at step 0.2; the dispersed length
  ceil(S + shift[0] * max DM) in float (src/DedispersionTest.cpp:129);
* 5 % of channels zapped by seed 7;
* uint8 samples rint(N(128, 20)) clipped to 0..255 (PCG64, seed 1 + rank),
  plus 20 dispersed pulses (DM uniform over the range, width 1-8, amplitude
  3-10 sigma, delay trunc(DM * shift)) drawn from the next seed.
"""
from __future__ import annotations

import math

import numpy as np

from . import row_bytes, shifts as oracle_shifts
from .types import DdObservation

f32 = np.float32


def observation(channels=1536, min_freq=1220.0, bandwidth=0.1953125, sampling_time=81.92e-6,
                samples=24576, dms=2048, first_dm=0.0, dm_step=0.2, padding=128):
    """(struct, shift table) of a one-beam single-step observation."""
    o = DdObservation()
    o.nr_beams = o.nr_synthesized_beams = o.nr_subbands = o.downsampling = 1
    o.nr_channels = channels
    o.nr_samples_per_batch = samples
    o.sampling_time = sampling_time
    o.min_freq = min_freq
    o.channel_bandwidth = bandwidth
    o.nr_dms, o.first_dm, o.dm_step = dms, first_dm, dm_step
    sh = oracle_shifts(o, padding)
    maxdm = f32(o.first_dm) + f32(dms - 1) * f32(o.dm_step)
    o.nr_samples_per_dispersed_batch = int(math.ceil(f32(f32(samples) +
                                                         f32(f32(sh[0]) * f32(maxdm)))))
    return o, sh


def zapped(channels: int, fraction: float, seed: int, padding: int) -> np.ndarray:
    """uint32 mask, round(fraction * channels) channels set, padded to padding/4."""
    q = padding // 4 or 1
    z = np.zeros(-(-channels // q) * q, np.uint32)
    k = int(round(fraction * channels))
    if k:
        z[np.random.default_rng(seed).choice(channels, size=k, replace=False)] = 1
    return z


def _pulses(vals: np.ndarray, sh: np.ndarray, o: DdObservation, count: int, sigma: float,
            seed: int) -> None:
    rng = np.random.default_rng(seed)
    nch = vals.shape[1]
    hi = o.first_dm + (o.nr_dms - 1) * o.dm_step
    for _ in range(count):
        dm = float(rng.uniform(o.first_dm, hi))
        t = int(rng.integers(0, max(1, o.nr_samples_per_batch - 8)))
        width = int(rng.integers(1, 9))
        amp = int(round(float(rng.uniform(3.0, 10.0)) * sigma))
        delay = np.floor(f32(dm) * sh[:nch].astype(f32)).astype(np.int64)
        for c in range(nch):
            s0 = t + delay[c]
            seg = vals[:, c, s0:s0 + width].astype(np.int64) + amp
            vals[:, c, s0:s0 + width] = np.minimum(seg, 255).astype(np.uint8)


def single_step(seed: int = 1, padding: int = 128, pulses: int = 20, mean: float = 128.0,
                sigma: float = 20.0):
    """(observation, shifts, zapped, mapping, input bytes) of the benchmark's
    single-step workload for beam seed ``seed``."""
    o, sh = observation(padding=padding)
    z = zapped(o.nr_channels, 0.05, 7, padding)
    q = padding // 4 or 1
    mapping = np.zeros(-(-o.nr_channels // q) * q, np.uint32)
    n = o.nr_samples_per_dispersed_batch
    rng = np.random.default_rng(seed)
    vals = np.clip(np.rint(rng.normal(mean, sigma, size=(1, o.nr_channels, n))), 0,
                   255).astype(np.uint8)
    if pulses:
        _pulses(vals, sh, o, pulses, sigma, seed + 1)
    inp = np.zeros((1, o.nr_channels, row_bytes(n, 8, padding)), np.uint8)
    inp[..., :n] = vals
    return o, sh, z, mapping, inp.reshape(-1)
