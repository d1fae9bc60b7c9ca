"""Seeded synthetic filterbank workloads.

No public dataset is used by the reference's tests or benchmarks; every input
here is drawn from numpy's PCG64 generator with a fixed seed, so the same
bytes come out on any machine.  Shapes and value distributions follow the
workloads the engine is measured on:

* :func:`small_observation` -- 256 channels of 0.1953125 MHz from 1425 MHz,
  40.96 us sampling, 1024 samples per batch, 128 DMs from 0 at step 0.25,
  uint8 from a Gaussian of mean 128 and sigma 16, no zapped channels.
* :func:`large_observation` -- 1536 channels of 0.1953125 MHz from 1220 MHz,
  81.92 us sampling, 24576 samples per batch, 2048 DMs from 0 at step 0.2,
  uint8 Gaussian noise (mean 128, sigma 20) with 20 injected dispersed pulses,
  5 % of channels zapped; in subband mode 32 subbands, 64 step-one DMs at
  step 6.4 and 32 step-two DMs at step 0.2.

The dispersed batch length follows src/DedispersionTest.cpp:129 (single
step) and :145-146 (step one, two): ceil(S + shift[0] * max DM) in float.
"""
from __future__ import annotations

import math

import numpy as np

from . import DD_SINGLE_STEP, DD_STEP_ONE, DD_STEP_TWO, Observation, getShifts, getShiftsStepTwo
from . import layout as _layout

f32 = np.float32


def dispersed_samples(samples: int, shift0: float, first: float, nr: int, step: float) -> int:
    """ceil(S + shift0 * (first + (nr - 1) * step)) in float arithmetic."""
    maxdm = f32(first) + f32(nr - 1) * f32(step)
    return int(math.ceil(f32(f32(samples) + f32(f32(shift0) * f32(maxdm)))))


def make_observation(channels: int, min_freq: float, bandwidth: float, sampling_time: float,
                     samples: int, dms: int, first_dm: float, dm_step: float, *, beams: int = 1,
                     synthesized_beams: int = 1, subbands: int = 0, dms1: int = 0,
                     first_dm1: float = 0.0, dm_step1: float = 0.0,
                     padding: int = 0) -> Observation:
    """An Observation with the dispersed lengths set as DedispersionTest sets them.
    ``subbands > 0`` also fills the step-one fields (S1, S1_disp, DM range)."""
    o = Observation()
    o.setNrBeams(beams)
    o.setNrSynthesizedBeams(synthesized_beams)
    o.setNrSamplesPerBatch(samples)
    o.setSamplingTime(sampling_time)
    o.setFrequencyRange(subbands if subbands else 1, channels, min_freq, bandwidth)
    o.setDMRange(dms, first_dm, dm_step)
    shifts = getShifts(o, padding)
    o.setNrSamplesPerDispersedBatch(dispersed_samples(samples, shifts[0], first_dm, dms, dm_step))
    if subbands:
        o.setDMRange(dms1, first_dm1, dm_step1, True)
        sh2 = getShiftsStepTwo(o, padding)
        s1 = dispersed_samples(samples, sh2[0], first_dm, dms, dm_step)
        o.setNrSamplesPerBatch(s1, True)
        o.setNrSamplesPerDispersedBatch(dispersed_samples(s1, shifts[0], first_dm1, dms1,
                                                          dm_step1), True)
    return o


def small_observation(padding: int = 0) -> Observation:
    return make_observation(256, 1425.0, 0.1953125, 40.96e-6, 1024, 128, 0.0, 0.25,
                            padding=padding)


def large_observation(padding: int = 0, subbands: bool = False) -> Observation:
    if subbands:
        return make_observation(1536, 1220.0, 0.1953125, 81.92e-6, 24576, 32, 0.0, 0.2,
                                subbands=32, dms1=64, first_dm1=0.0, dm_step1=6.4,
                                padding=padding)
    return make_observation(1536, 1220.0, 0.1953125, 81.92e-6, 24576, 2048, 0.0, 0.2,
                            padding=padding)


def pack_subbyte(values: np.ndarray, bits: int, row_bytes: int) -> np.ndarray:
    """Pack the last axis (one sample per element, < 2**bits) LSB-first:
    sample k goes to byte k // (8 // bits) at bit (k % (8 // bits)) * bits."""
    per = 8 // bits
    lead = values.shape[:-1]
    n = values.shape[-1]
    padded = np.zeros(lead + (row_bytes * per,), dtype=np.uint8)
    padded[..., :n] = values
    grouped = padded.reshape(lead + (row_bytes, per)).astype(np.uint16)
    shifts = (np.arange(per, dtype=np.uint16) * bits)
    return (grouped << shifts).sum(axis=-1).astype(np.uint8)


def unpack_subbyte(packed: np.ndarray, bits: int, samples: int) -> np.ndarray:
    per = 8 // bits
    shifts = (np.arange(per, dtype=np.uint8) * bits)
    vals = (packed[..., None] >> shifts) & ((1 << bits) - 1)
    return vals.reshape(packed.shape[:-1] + (-1,))[..., :samples].astype(np.uint8)


def zapped_mask(channels: int, fraction: float, seed: int, padding: int = 0) -> np.ndarray:
    """uint32 mask (nonzero = zapped) with round(fraction * C) channels zapped."""
    n = channels if padding == 0 else -(-channels // (padding // 4 or 1)) * (padding // 4 or 1)
    z = np.zeros(n, dtype=np.uint32)
    k = int(round(fraction * channels))
    if k:
        rng = np.random.default_rng(seed)
        z[rng.choice(channels, size=k, replace=False)] = 1
    return z


def identity_mapping(obs: Observation, padding: int, subbands: bool = False) -> np.ndarray:
    """AstroData::generateBeamMapping: synthesized beam b reads beam b % nrBeams."""
    n = obs.getNrSubbands() if subbands else obs.getNrChannels()
    row = n if padding == 0 else -(-n // (padding // 4 or 1)) * (padding // 4 or 1)
    m = np.zeros((obs.getNrSynthesizedBeams(), row), dtype=np.uint32)
    for b in range(obs.getNrSynthesizedBeams()):
        m[b, :] = b % max(1, obs.getNrBeams())
    return m.reshape(-1)


def gaussian_rows(rng: np.random.Generator, shape, mean: float, sigma: float,
                  maxval: int) -> np.ndarray:
    x = rng.normal(mean, sigma, size=shape)
    return np.clip(np.rint(x), 0, maxval).astype(np.uint16 if maxval > 255 else np.uint8)


def inject_pulses(values: np.ndarray, shifts: np.ndarray, samples: int, first_dm: float,
                  dm_step: float, nr_dms: int, count: int, sigma: float, seed: int,
                  zapped: np.ndarray | None = None, maxval: int = 255) -> list[dict]:
    """Add ``count`` dispersed pulses in place to values[beam, channel, sample];
    each has a DM uniform over the trial range, a width of 1-8 samples and an
    amplitude of 3-10 sigma, delayed per channel by trunc(DM * shift)."""
    rng = np.random.default_rng(seed)
    C = values.shape[1]
    pulses = []
    maxdm = first_dm + (nr_dms - 1) * dm_step
    for _ in range(count):
        dm = float(rng.uniform(first_dm, maxdm))
        t = int(rng.integers(0, max(1, samples - 8)))
        width = int(rng.integers(1, 9))
        amp = int(round(float(rng.uniform(3.0, 10.0)) * sigma))
        delays = np.floor(f32(dm) * shifts[:C].astype(f32)).astype(np.int64)
        for c in range(C):
            s0 = t + delays[c]
            seg = values[:, c, s0:s0 + width].astype(np.int64) + amp
            values[:, c, s0:s0 + width] = np.minimum(seg, maxval).astype(values.dtype)
        pulses.append({"dm": dm, "t": t, "width": width, "amplitude": amp})
    return pulses


def make_input(obs: Observation, bits: int, padding: int, seed: int, *, mode: int = DD_SINGLE_STEP,
               mean: float = 128.0, sigma: float = 20.0, distribution: str = "gaussian",
               pulses: int = 0, shifts: np.ndarray | None = None) -> np.ndarray:
    """Input buffer in the reference layout for ``mode`` (flat, bytes for
    bits <= 8, else uint16/float32 elements).

    distribution: "gaussian" (mean, sigma, clipped to the type's range),
    "uniform" (full bit range), "constant" (every sample = mean)."""
    rng = np.random.default_rng(seed)
    lay = _layout(obs, mode, bits if mode != DD_STEP_TWO else 32, padding)
    if mode == DD_STEP_TWO:
        rows = obs.getNrBeams() * obs.getNrDMs(True) * obs.getNrSubbands()
        n = obs.getNrSamplesPerBatch(True)
        elems = lay.input_row_bytes // 4
        out = np.zeros((rows, elems), dtype=np.float32)
        if distribution == "constant":
            out[:, :n] = mean
        else:
            out[:, :n] = rng.integers(0, 10, size=(rows, n)).astype(np.float32)
        return out.reshape(-1)
    sub = mode == DD_STEP_ONE
    samples = obs.getNrSamplesPerDispersedBatch(sub)
    B, Cn = obs.getNrBeams(), obs.getNrChannels()
    maxval = (1 << bits) - 1 if bits <= 16 else 0
    if bits == 32:
        vals = rng.normal(mean, sigma, size=(B, Cn, samples)).astype(np.float32)
        if distribution == "constant":
            vals[:] = mean
        elems = lay.input_row_bytes // 4
        out = np.zeros((B, Cn, elems), dtype=np.float32)
        out[..., :samples] = vals
        return out.reshape(-1)
    if distribution == "gaussian":
        vals = gaussian_rows(rng, (B, Cn, samples), mean, sigma, maxval)
    elif distribution == "uniform":
        vals = rng.integers(0, maxval + 1, size=(B, Cn, samples)).astype(
            np.uint16 if bits > 8 else np.uint8)
    elif distribution == "constant":
        vals = np.full((B, Cn, samples), int(mean), dtype=np.uint16 if bits > 8 else np.uint8)
    else:
        raise ValueError(distribution)
    if pulses:
        sh = shifts if shifts is not None else getShifts(obs, padding)
        inject_pulses(vals, sh, obs.getNrSamplesPerBatch(sub), obs.getFirstDM(sub),
                      obs.getDMStep(sub), obs.getNrDMs(sub), pulses, sigma, seed + 1,
                      maxval=maxval)
    if bits < 8:
        return pack_subbyte(vals, bits, int(lay.input_row_bytes)).reshape(-1)
    if bits == 8:
        out = np.zeros((B, Cn, lay.input_row_bytes), dtype=np.uint8)
        out[..., :samples] = vals
        return out.reshape(-1)
    elems = lay.input_row_bytes // 2
    out = np.zeros((B, Cn, elems), dtype=np.uint16)
    out[..., :samples] = vals
    return out.reshape(-1)


def batched_shapes(count: int = 40, seed: int = 2024) -> list[dict]:
    """Uneven beams for one batched launch: channels in {384, 1536} over the
    same 300 MHz band from 1220 MHz, samples uniform over 8192-32768 in steps of
    1024, DMs uniform over 512-4096 in steps of 128, DM step uniform over
    0.1-0.5, input bits in {2, 4, 8}; 81.92 us sampling."""
    rng = np.random.default_rng(seed)
    shapes = []
    for i in range(count):
        ch = int(rng.choice([384, 1536]))
        shapes.append({
            "channels": ch,
            "bandwidth": 300.0 / ch,
            "samples": int(rng.integers(8, 33)) * 1024,
            "dms": int(rng.integers(4, 33)) * 128,
            "dm_step": float(np.float32(rng.uniform(0.1, 0.5))),
            "bits": int(rng.choice([2, 4, 8])),
            "seed": seed * 1000 + i,
        })
    return shapes


def shape_observation(shape: dict, padding: int) -> Observation:
    return make_observation(shape["channels"], 1220.0, shape["bandwidth"], 81.92e-6,
                            shape["samples"], shape["dms"], 0.0, shape["dm_step"],
                            padding=padding)


def device_uniform_input(torch, obs: Observation, bits: int, padding: int, seed: int):
    """Seeded input on the GPU, uniform over the full bit range, packed
    LSB-first for sub-byte widths, in the single-step row layout."""
    lay = _layout(obs, DD_SINGLE_STEP, bits, padding)
    C_, n = obs.getNrChannels(), obs.getNrSamplesPerDispersedBatch()
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    vals = torch.randint(0, 1 << bits, (C_, n), generator=g, device="cuda", dtype=torch.int32)
    row = int(lay.input_row_bytes)
    buf = torch.zeros((obs.getNrBeams() * C_, row), dtype=torch.uint8, device="cuda")
    if bits == 8:
        buf[:C_, :n] = vals.to(torch.uint8)
    else:
        per = 8 // bits
        m = -(-n // per) * per
        padded = torch.zeros((C_, m), dtype=torch.int32, device="cuda")
        padded[:, :n] = vals
        shifts = (torch.arange(per, device="cuda", dtype=torch.int32) * bits)
        packed = (padded.view(C_, m // per, per) << shifts).sum(dim=2).to(torch.uint8)
        buf[:C_, :m // per] = packed
    return buf.view(-1)


def output_buffer(obs: Observation, mode: int, padding: int, bits: int = 8) -> np.ndarray:
    lay = _layout(obs, mode, bits if mode != DD_STEP_TWO else 32, padding)
    return np.zeros(lay.output_bytes // 4, dtype=np.float32)
