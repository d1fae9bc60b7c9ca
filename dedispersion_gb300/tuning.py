"""Autotuning of the tile configuration: an exhaustive sweep and a learned
cost model that times only its top candidates.

* :func:`sweep` is the engine's DedispersionTuning (src/DedispersionTuning.cpp):
  every compiled configuration of the input width's kernel family is run on
  the problem and timed with CUDA events inside the library (dd_plan_time);
  results carry the reference's GFLOP/s figure, 1e-9 * beams * DMs *
  (channels - zapped) * samples / time (src/DedispersionTuning.cpp:327,
  412-425).  ``python -m dedispersion_gb300.tuning`` takes the reference's
  switches and prints its row format, or with -best the tuned-conf line
  "nrDMs split local unroll tD0 tD1 tD2 iD0 iD1 iD2" (:416-437), which
  readTunedDedispersionConf reads.
* :class:`LearnedTuner` predicts log(time per DM-sample) of every configuration
  from shape and configuration features with the library's CUDA MLP
  (dedispersion_gb300.costmodel), then times only the top k.  The sweep stays
  the arbiter of what is fastest; the model never touches outputs.  A trained model is saved and
  loaded (``LearnedTuner.save`` / ``load``); on the command line
  ``-train_model model.npz`` sweeps the seeded study shapes and saves one, and
  ``-learned model.npz -top_k k`` times only the model's top k of a problem
  (single step and step one; step two keeps the full sweep).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import functools
import math
import sys
import time
from dataclasses import dataclass, field

import numpy as np

from . import (DD_SINGLE_STEP, DD_STEP_ONE, DD_STEP_TWO, DedispersionConf, Plan, getShifts,
               kernels, layout)
from . import synthetic as syn
from ._abi import check, lib

import ctypes as C


# ---------------------------------------------------------------------------
# exhaustive sweep

@dataclass
class TuneResult:
    kernel: int
    name: str
    conf: DedispersionConf
    mean_ms: float
    std_ms: float
    gflops: float
    wall_s: float  # tuning wall time spent on this configuration


def family_kernels(mode: int, bits: int):
    """Compiled configurations for a mode and input width; the
    shared-partial-sum ones (items_d2 = 8) and the TMEM-window one
    (items_d2 = 3) compute single-step input only."""
    fam = 32 if mode == DD_STEP_TWO else (8 if bits <= 8 else bits)
    return [k for k in kernels() if k.elem_bits == fam and
            (mode == DD_SINGLE_STEP or k.conf.getNrItemsD2() not in (8, 3))]


def _time_plan(plan: Plan, d_in, d_out, warmup: int, iterations: int):
    mean, std = C.c_float(0), C.c_float(0)
    check(lib().dd_plan_time(plan._h, C.c_void_p(int(d_in.data_ptr())),
                             C.c_void_p(int(d_out.data_ptr())), warmup, iterations,
                             C.byref(mean), C.byref(std)))
    return mean.value, std.value


def work_units(obs, mode: int, live: int) -> float:
    """beams x DMs x live rows x samples: the reference tuner's FLOP count."""
    if mode == DD_SINGLE_STEP:
        return obs.getNrSynthesizedBeams() * obs.getNrDMs() * live * obs.getNrSamplesPerBatch()
    if mode == DD_STEP_ONE:
        return obs.getNrBeams() * obs.getNrDMs(True) * live * obs.getNrSamplesPerBatch(True)
    return (obs.getNrSynthesizedBeams() * obs.getNrDMs(True) * obs.getNrDMs() *
            obs.getNrSubbands() * obs.getNrSamplesPerBatch())


def sweep(obs, mode: int, bits: int, padding: int, shifts, zapped=None, mapping=None,
          d_in=None, d_out=None, warmup: int = 1, iterations: int = 3, device: int = 0,
          candidates=None) -> list[TuneResult]:
    """Time every configuration in `candidates` (default: the whole family)."""
    import torch
    lay = layout(obs, mode, bits if mode != DD_STEP_TWO else 32, padding)
    if d_in is None:
        d_in = torch.randint(0, 255, (lay.input_bytes,), dtype=torch.uint8,
                             device=f"cuda:{device}")
        if mode == DD_STEP_TWO or bits == 32:
            d_in = torch.rand(lay.input_bytes // 4, device=f"cuda:{device}")
    if d_out is None:
        d_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32, device=f"cuda:{device}")
    n = obs.getNrChannels() if mode != DD_STEP_TWO else obs.getNrSubbands()
    live = n if zapped is None else int((np.asarray(zapped)[:n] == 0).sum())
    units = work_units(obs, mode, live)
    out = []
    from . import DedispersionError
    from ._abi import DD_ERR_INVALID_ARGUMENT, DD_ERR_UNSUPPORTED
    for k in (candidates if candidates is not None else family_kernels(mode, bits)):
        t0 = time.perf_counter()
        try:
            plan = Plan(obs, mode, bits, padding, device=device, kernel=k.index)
        except DedispersionError as e:
            if e.status == DD_ERR_UNSUPPORTED:
                continue
            raise
        try:
            plan.setShifts(shifts)
            if mode != DD_STEP_TWO and zapped is not None:
                plan.setZappedChannels(zapped)
            if mode != DD_STEP_ONE:
                plan.setBeamMapping(mapping if mapping is not None
                                    else np.zeros(obs.getNrSynthesizedBeams() *
                                                  lay.mapping_row_elems, np.uint32))
            mean, std = _time_plan(plan, d_in, d_out, warmup, iterations)
        except DedispersionError as e:
            # a configuration this problem cannot run (e.g. its window does
            # not fit in shared memory) is skipped, as the reference's tuner
            # skips configurations that fail (src/DedispersionTuning.cpp:396-409)
            if e.status in (DD_ERR_UNSUPPORTED, DD_ERR_INVALID_ARGUMENT):
                continue
            raise
        finally:
            plan.close()
        out.append(TuneResult(k.index, k.name, k.conf, mean, std, 1e-9 * units / (mean * 1e-3),
                              time.perf_counter() - t0))
    out.sort(key=lambda r: r.mean_ms)
    return out


# Configurations a batch times per beam before it commits: every
# shared-partial-sum tile and the direct tiles that win on some of the
# batched workload's beams (wide channels, large DM steps).
BATCH_SHORTLIST = ("shared8_", "swar8_i4_d4_w8_c16_vkUnpackPermuteMad",
                   "swar8_i4_d4_w16_c16_vkUnpackPermuteMad",
                   "swar8_i2_d8_w8_c16_vkUnpackPermuteMad")


def batch_candidates():
    """The shortlist of 1-8-bit single-step configurations a batch tunes over."""
    return [k for k in kernels() if k.elem_bits == 8 and
            any(k.name.startswith(n) if n.endswith("_") else k.name == n
                for n in BATCH_SHORTLIST)]


def pick(obs, bits: int, padding: int, shifts, zapped, mapping, d_in, d_out, candidates=None,
         iterations: int = 3, device: int = 0) -> TuneResult:
    """The fastest of `candidates` (default: :func:`batch_candidates`) on one
    single-step problem, timed on its own device buffers."""
    res = sweep(obs, DD_SINGLE_STEP, bits, padding, shifts, zapped, mapping, d_in, d_out,
                iterations=iterations, device=device,
                candidates=candidates if candidates is not None else batch_candidates())
    if not res:
        raise ValueError("no candidate configuration runs this problem")
    return res[0]


# ---------------------------------------------------------------------------
# learned tuning

BITS = (2, 4, 8, 32)
VARIANTS = ("PermuteMad", "Permute", "PermuteHalf", "MaskHigh")  # swar8 name suffixes
FAMILIES = ("swar8", "scalar", "shared8", "tmem32")                 # name prefixes
# Delay per unit DM of the lowest channel, in samples, for the study band
# (1220-1520 MHz at 81.92 us); the window spread of a tile scales with it.
STUDY_SHIFT0 = 12.1


@dataclass
class Shape:
    """One tuning problem: geometry, input width and subbands (0: single step)."""

    channels: int
    dms: int
    samples: int
    bits: int
    subbands: int
    dm_step: float = 0.2
    seed: int = 0
    shift0: float = 0.0  # delay per unit DM of the lowest channel (0: the study band's)

    def mode(self) -> int:
        return DD_STEP_ONE if self.subbands else DD_SINGLE_STEP


def study_shapes(count: int = 400, seed: int = 4242) -> list[Shape]:
    """Seeded shapes over channels 256-4096, DMs 256-8192, samples 4096-65536,
    input bits 2/4/8/32, subbands 0/16/32/64/128."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        sb = int(rng.choice([0, 16, 32, 64, 128]))
        ch = int(2 ** rng.uniform(8, 12))
        if sb:
            ch = max(sb * 2, ch // sb * sb)
        out.append(Shape(channels=ch, dms=int(2 ** rng.uniform(8, 13)) // 32 * 32 or 32,
                         samples=int(2 ** rng.uniform(12, 16)) // 1024 * 1024,
                         bits=int(rng.choice(BITS)), subbands=sb,
                         dm_step=float(np.float32(rng.uniform(0.05, 0.5))), seed=seed + i))
    return out


def measured_observation(s: Shape, padding: int, max_dms: int = 1024,
                         max_samples: int = 16384):
    """The shape's observation cut to at most max_dms DM trials (per step) and
    max_samples samples, keeping channels, DM step and input width: the
    per-DM-sample cost of a tile depends on those and on how the tiles fill
    the GPU's waves (a feature of its own), not on the trial count as such.
    The cut keeps several waves of tiles for most configurations."""
    S = min(s.samples, max_samples)
    bw = 300.0 / s.channels
    if s.subbands:
        d1 = max(1, min(s.dms // 32, max_dms // 4))
        return syn.make_observation(s.channels, 1220.0, bw, 81.92e-6, S, 32, 0.0, s.dm_step,
                                    subbands=s.subbands, dms1=d1, first_dm1=0.0,
                                    dm_step1=s.dm_step * 32, padding=padding)
    return syn.make_observation(s.channels, 1220.0, bw, 81.92e-6, S, min(s.dms, max_dms), 0.0,
                                s.dm_step, padding=padding)


FEATURE_NAMES = ("log2 channels", "log2 rows", "log2 dms", "log2 samples", "log2 subbands+1",
                 "log2 spread", "log2 sharing", "log2 items d0", "log2 items d1",
                 "log2 warps d1", "log2 unroll", "log2 tile dms", "log2 tile samples",
                 "subband", "log2 waves", "wave efficiency", "short groups",
                 "log2 shared adds ratio") + \
    tuple(f"bits {b}" for b in BITS) + \
    tuple(f"variant {v}" for v in VARIANTS) + tuple(f"family {f}" for f in FAMILIES)


GPU_SMS = 152  # SMs of a GB300


@functools.lru_cache(maxsize=4096)
def shared_adds_ratio(channels: int, dms: int, dm_step: float, tile_d: int,
                      samples_sub: int = 12, samples_tile: int = 4) -> float:
    """Estimated integer adds of the shared-partial-sum tile per direct-sum
    add, for a single-step shape of the study band (1220-1520 MHz at 81.92
    us): rows in subgroups of 8, per DM tile each distinct relative-delay
    vector of a subgroup summed once (its first vector over its 8 rows, each
    next one from the previous with 2 adds per moved row, in DM order) and
    one series add per DM and subgroup.  Evaluated on `samples_sub` subgroups
    x `samples_tile` DM tiles spread over the shape (about a millisecond), in
    the reference's float order for the delays."""
    bw = 300.0 / channels
    f = 1220.0 + np.arange(channels, dtype=np.float64) * bw
    shift = (4148.808 * (1.0 / f ** 2 - 1.0 / f[-1] ** 2) / 81.92e-6).astype(np.float32)
    dms = max(1, min(dms, 1024))
    nsub = max(1, channels // 8)
    tiles = max(1, -(-dms // tile_d))
    subs = np.unique(np.linspace(0, nsub - 1, min(nsub, samples_sub)).astype(int))
    tl = np.unique(np.linspace(0, tiles - 1, min(tiles, samples_tile)).astype(int))
    rows = shift[(8 * subs[:, None] + np.arange(8)[None, :]).clip(max=channels - 1)]  # [g, 8]
    weights = (np.int64(1) << (np.arange(8, dtype=np.int64) * 7))
    cost = 0.0
    for t in tl:
        dm = np.minimum(np.arange(t * tile_d, (t + 1) * tile_d), dms - 1).astype(np.float32)
        val = (dm * np.float32(dm_step)).astype(np.float32)
        d = (rows[:, :, None] * val[None, None, :]).astype(np.float32).astype(np.int64)
        rel = d - d.min(axis=1, keepdims=True)                                # [g, 8, D]
        keys = (np.minimum(rel, 127) * weights[None, :, None]).sum(axis=1)  # [g, D]
        for gi in range(len(subs)):
            _, first = np.unique(keys[gi], return_index=True)
            v = rel[gi][:, np.sort(first)]                                   # distinct, DM order
            moves = int((v[:, 1:] != v[:, :-1]).sum())
            cost += (8 + 2 * moves) / (8 * tile_d)
    return float(1.0 / 8 + cost / (len(tl) * len(subs)))


def resident_ctas(name: str, conf: DedispersionConf) -> int:
    """CTAs of a configuration resident per SM, as its kernel's launch bounds
    budget them (dd_kernels.cuh): the shared and TMEM-window tiles one, the
    others one to four by warps per CTA."""
    warps = conf.nrThreadsD1
    if name.startswith(("shared8", "tmem32")):
        return 1
    if name.startswith("swar8"):
        return 1 if warps >= 16 else (2 if warps >= 8 else 4)
    return 2 if warps >= 8 else 4


def features(s: Shape, conf: DedispersionConf, name: str) -> np.ndarray:
    """Shape and configuration features of one (problem, configuration) pair."""
    shift0 = s.shift0 or STUDY_SHIFT0
    tile_d = conf.nrThreadsD1 * conf.nrItemsD1
    spread = shift0 * s.dm_step * (32 if s.subbands else 1) * tile_d
    rows = s.channels // s.subbands if s.subbands else s.channels
    # Relative-delay growth across eight adjacent rows over the tile's DMs:
    # how often rows share a delay vector (the shared-partial-sum family's gain).
    share = shift0 * s.dm_step * (32 if s.subbands else 1) * tile_d * 8 / max(1, rows)
    # Waves of tiles on the GPU: tiles / (SMs x resident CTAs per SM), and
    # how full the last wave is.
    tile_t = 32 * conf.nrItemsD0
    dm_count = max(1, s.dms // 32) if s.subbands else max(1, s.dms)
    tiles = (max(1, s.subbands) * -(-max(1, s.samples) // tile_t) * -(-dm_count // tile_d))
    waves = tiles / (GPU_SMS * resident_ctas(name, conf))
    f = [math.log2(s.channels), math.log2(rows), math.log2(max(1, s.dms)),
         math.log2(max(1, s.samples)), math.log2(s.subbands + 1), math.log2(1 + spread),
         math.log2(1 + share),
         math.log2(conf.nrItemsD0), math.log2(conf.nrItemsD1), math.log2(conf.nrThreadsD1),
         math.log2(conf.unroll), math.log2(tile_d), math.log2(tile_t),
         float(s.subbands > 0), math.log2(1 + waves), waves / math.ceil(waves),
         float(name.startswith("swar8s")),
         math.log2(shared_adds_ratio(s.channels, s.dms, s.dm_step, tile_d))
         if name.startswith("shared8") else 0.0]
    f += [float(s.bits == b) for b in BITS]
    f += [float(name.endswith("_vkUnpack" + v)) for v in VARIANTS]
    f += [float(name.startswith(fam)) for fam in FAMILIES]
    return np.array(f, np.float32)


@dataclass
class StudyRecord:
    shape: Shape
    results: list  # TuneResult, all configurations of the family
    units: float   # DM-samples of the measured problem


def collect(shapes: list[Shape], padding: int = 128, iterations: int = 3, device: int = 0,
            log=None, full_size: bool = False) -> list[StudyRecord]:
    """Time every configuration of every shape (the exhaustive sweep), each
    cut as measured_observation cuts it, or at its full size."""
    import torch
    records = []
    for i, s in enumerate(shapes):
        obs = (measured_observation(s, padding, max_dms=s.dms, max_samples=s.samples)
               if full_size else measured_observation(s, padding))
        mode = s.mode()
        shifts = getShifts(obs, padding)
        zapped = syn.zapped_mask(s.channels, 0.05, s.seed, padding)
        lay = layout(obs, mode, s.bits, padding)
        g = torch.Generator(device=f"cuda:{device}")
        g.manual_seed(s.seed)
        if s.bits == 32:
            d_in = torch.rand(lay.input_bytes // 4, generator=g, device=f"cuda:{device}")
        elif s.bits == 16:
            d_in = torch.randint(0, 60000, (lay.input_bytes // 2,), generator=g,
                                 device=f"cuda:{device}", dtype=torch.int32).to(torch.int16)
        else:
            d_in = torch.randint(0, 255, (lay.input_bytes,), generator=g, device=f"cuda:{device}",
                                 dtype=torch.uint8)
        d_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32, device=f"cuda:{device}")
        res = sweep(obs, mode, s.bits, padding, shifts, zapped, None, d_in, d_out,
                    iterations=iterations, device=device)
        units = (obs.getNrDMs(True) * obs.getNrSubbands() * obs.getNrSamplesPerBatch(True)
                 if s.subbands else obs.getNrDMs() * obs.getNrSamplesPerBatch())
        # the record describes the problem that was timed
        timed = dataclasses.replace(
            s, dms=obs.getNrDMs(True) * 32 if s.subbands else obs.getNrDMs(),
            samples=obs.getNrSamplesPerBatch())
        records.append(StudyRecord(timed, res, units))
        if log and (i % 20 == 0):
            log(f"shape {i}/{len(shapes)}: {s} best {res[0].name} {res[0].mean_ms:.3f} ms")
    return records


def dataset(records: list[StudyRecord]):
    X, y, owner = [], [], []
    for r_i, rec in enumerate(records):
        for res in rec.results:
            X.append(features(rec.shape, res.conf, res.name))
            y.append(math.log(res.mean_ms * 1e-3 / rec.units))
            owner.append(r_i)
    return np.stack(X), np.array(y, np.float32), np.array(owner)


class LearnedTuner:
    """MLP over (shape, configuration) features, trained on measured timings;
    `members` > 1 trains that many networks from different seeds and
    averages their predictions (an ensemble ranks more steadily than one
    network, whose training order on the GPU is not deterministic)."""

    def __init__(self, hidden: int = 128, layers: int = 3, seed: int = 0, device: int = 0,
                 members: int = 1):
        self.hidden, self.layers, self.seed, self.device = hidden, layers, seed, device
        self.members = members
        self.models = []
        self.mu = self.sd = None
        self.train_loss = None

    @property
    def model(self):
        return self.models[0] if self.models else None

    def fit(self, X: np.ndarray, y: np.ndarray, steps: int = 3000, lr: float = 1e-3) -> float:
        from .costmodel import MLP
        self.mu, self.sd = X.mean(axis=0), X.std(axis=0) + 1e-6
        self.ymu, self.ysd = float(y.mean()), float(y.std() + 1e-6)
        self.models, losses = [], []
        for m in range(self.members):
            net = MLP(X.shape[1], self.hidden, self.layers, self.seed + m, self.device)
            losses.append(net.train((X - self.mu) / self.sd, (y - self.ymu) / self.ysd,
                                    steps, lr))
            self.models.append(net)
        self.train_loss = float(np.mean(losses))
        return self.train_loss

    def predict(self, X: np.ndarray) -> np.ndarray:
        Xn = (X - self.mu) / self.sd
        return np.mean([net.forward(Xn) for net in self.models], axis=0) * self.ysd + self.ymu

    def rank(self, shape: Shape, candidates) -> list:
        X = np.stack([features(shape, k.conf, k.name) for k in candidates])
        order = np.argsort(self.predict(X))
        return [candidates[i] for i in order]

    def save(self, path: str) -> None:
        """Weights and normalisation, to rank new shapes without retraining."""
        np.savez(path, params=np.stack([net.params() for net in self.models]), mu=self.mu,
                 sd=self.sd, ymu=self.ymu, ysd=self.ysd, hidden=self.hidden, layers=self.layers,
                 features=len(self.mu), feature_names=np.array(FEATURE_NAMES))

    @classmethod
    def load(cls, path: str, device: int = 0) -> "LearnedTuner":
        from .costmodel import MLP
        z = np.load(path)
        if list(z["feature_names"]) != list(FEATURE_NAMES):
            raise ValueError(f"{path} was trained on other features; retrain it")
        params = np.atleast_2d(z["params"])
        t = cls(hidden=int(z["hidden"]), layers=int(z["layers"]), device=device,
                members=len(params))
        t.mu, t.sd = z["mu"], z["sd"]
        t.ymu, t.ysd = float(z["ymu"]), float(z["ysd"])
        for p in params:
            net = MLP(int(z["features"]), t.hidden, t.layers, 0, device)
            net.set_params(p)
            t.models.append(net)
        return t


def observation_shape(obs, mode: int, bits: int, shifts) -> Shape:
    """The learned tuner's view of a single-step or step-one problem."""
    shift0 = float(np.asarray(shifts)[0])
    if mode == DD_STEP_ONE:
        # the study's subband shapes take coarse steps of 32 fine ones
        return Shape(channels=obs.getNrChannels(), dms=obs.getNrDMs(True) * 32,
                     samples=obs.getNrSamplesPerBatch(True), bits=bits,
                     subbands=obs.getNrSubbands(), dm_step=obs.getDMStep(True) / 32,
                     shift0=shift0)
    return Shape(channels=obs.getNrChannels(), dms=obs.getNrDMs(),
                 samples=obs.getNrSamplesPerBatch(), bits=bits, subbands=0,
                 dm_step=obs.getDMStep(), shift0=shift0)


def train_model(path: str, count: int = 400, steps: int = 3000, device: int = 0,
                log=None) -> dict:
    """Sweep `count` seeded study shapes, train the cost model on all of them
    and save it (LearnedTuner.load reads it back)."""
    records = collect(study_shapes(count), device=device, log=log)
    X, y, _ = dataset(records)
    tuner = LearnedTuner(device=device)
    loss = tuner.fit(X, y, steps=steps)
    tuner.save(path)
    return {"shapes": count, "rows": int(len(y)), "train_loss_normalised": loss, "path": path}


def evaluate(records, tuner: LearnedTuner, test_idx, k: int = 2, seed: int = 7) -> dict:
    """Top-k by model, k random and the default configuration against the
    exhaustive best on held-out shapes; tuning wall time with and without."""
    rng = np.random.default_rng(seed)
    model_r, random_r, default_r, within5 = [], [], [], 0
    t_exhaustive = t_learned = 0.0
    per_shape = []
    for i in test_idx:
        rec = records[i]
        by_index = {r.kernel: r for r in rec.results}
        best = rec.results[0].mean_ms
        cands = [kk for kk in kernels() if kk.index in by_index]
        t0 = time.perf_counter()
        ranked = tuner.rank(rec.shape, cands)[:k]
        infer = time.perf_counter() - t0
        chosen = min(by_index[c.index].mean_ms for c in ranked)
        per_shape.append({"best": rec.results[0].name, "best_ms": best,
                          "chosen": [c.name for c in ranked], "chosen_ms": chosen,
                          "ratio": best / chosen})
        model_r.append(best / chosen)
        within5 += best / chosen >= 0.95
        rnd = rng.choice(len(cands), size=min(k, len(cands)), replace=False)
        random_r.append(best / min(by_index[cands[j].index].mean_ms for j in rnd))
        default_r.append(best / by_index[cands[0].index].mean_ms)
        t_exhaustive += sum(r.wall_s for r in rec.results)
        t_learned += infer + sum(by_index[c.index].wall_s for c in ranked)
    return {"held_out_shapes": len(test_idx), "k": k,
            "top_k_vs_best_mean": float(np.mean(model_r)),
            "top_k_vs_best_median": float(np.median(model_r)),
            "top_k_vs_best_worst": float(np.min(model_r)),
            "shapes_within_5pct": int(within5),
            "random_k_vs_best_mean": float(np.mean(random_r)),
            "default_vs_best_mean": float(np.mean(default_r)),
            "tuning_time_exhaustive_s": t_exhaustive, "tuning_time_learned_s": t_learned,
            "tuning_time_ratio": t_learned / t_exhaustive if t_exhaustive else None,
            "per_shape": per_shape}


def study(count: int = 400, train_fraction: float = 0.8, steps: int = 3000, k: int = 2,
          device: int = 0, log=print) -> dict:
    """The full learned-tuning study: sweep, train on 80 %, evaluate on 20 %."""
    shapes = study_shapes(count)
    t0 = time.perf_counter()
    records = collect(shapes, device=device, log=log)
    t_collect = time.perf_counter() - t0
    rng = np.random.default_rng(1)
    perm = rng.permutation(len(records))
    n_train = int(round(train_fraction * len(records)))
    train_idx, test_idx = perm[:n_train], perm[n_train:]
    X, y, owner = dataset(records)
    mask = np.isin(owner, train_idx)
    tuner = LearnedTuner(device=device)
    t0 = time.perf_counter()
    loss = tuner.fit(X[mask], y[mask], steps=steps)
    t_train = time.perf_counter() - t0
    test_mask = np.isin(owner, test_idx)
    pred = tuner.predict(X[test_mask])
    rep = evaluate(records, tuner, test_idx, k=k)
    rep["by_k"] = {str(kk): {key: v for key, v in evaluate(records, tuner, test_idx, k=kk).items()
                             if key in ("top_k_vs_best_mean", "shapes_within_5pct",
                                        "tuning_time_ratio")} for kk in (1, 2, 3, 4, 6)}
    rep.update({"shapes": count, "configurations_per_shape": float(np.mean(
        [len(r.results) for r in records])), "train_rows": int(mask.sum()),
        "train_loss_normalised": loss,
        "held_out_rmse_log_time": float(np.sqrt(np.mean((pred - y[test_mask]) ** 2))),
        "collect_s": t_collect, "train_s": t_train,
        "network": "3 x 128 ReLU, bf16 weights, fp32 accumulation, trained by the library's "
                   "CUDA kernels (Adam, full batch)"})
    return rep


def direct_sum_adds(s: Shape) -> float:
    """Direct-sum adds of a shape at full size (its single-step work)."""
    return float(s.channels) * s.dms * s.samples


def bench_report(count: int = 400, k: int = 2, steps: int = 2000, device: int = 0,
                 full_shapes: int = 8, max_full_adds: float = 2e11, large_train: int = 120,
                 max_large_adds: float = 4e11, members: int = 3) -> dict:
    """The learned tuner measured for a benchmark line: the study's sweep of
    `count` seeded shapes (cut to <= 1024 DMs x 16384 samples), the model
    trained on 80 % of them, its top-k against the exhaustive best on the
    held-out 20 % (k = 1, 2, 4), and the same at full size on the
    1536-channel x 2048-DM x 24576-sample workload (single step and 32
    subbands) plus `full_shapes` held-out shapes of at most `max_full_adds`
    direct-sum adds, each swept exhaustively at full size.  `large_train`
    training shapes are also timed cut only to <= 4096 DMs x 32768 samples
    (at most `max_large_adds` direct-sum adds), so that the model sees how
    the configurations rank on large problems too."""
    t0 = time.perf_counter()
    shapes = study_shapes(count)
    records = collect(shapes, device=device)
    t_collect = time.perf_counter() - t0
    perm = np.random.default_rng(1).permutation(len(records))
    n_train = int(round(0.8 * len(records)))
    train_idx, test_idx = perm[:n_train], perm[n_train:]
    t0 = time.perf_counter()
    large = []
    for i in train_idx:
        s = shapes[i]
        cut = dataclasses.replace(s, dms=min(s.dms, 4096), samples=min(s.samples, 32768))
        if len(large) < large_train and direct_sum_adds(cut) <= max_large_adds:
            large.append(cut)
    large_records = collect(large, device=device, full_size=True)
    t_large = time.perf_counter() - t0
    X, y, owner = dataset(records + large_records)
    mask = np.isin(owner, train_idx) | (owner >= len(records))
    tuner = LearnedTuner(device=device, members=members)
    t0 = time.perf_counter()
    tuner.fit(X[mask], y[mask], steps=steps)
    t_train = time.perf_counter() - t0
    keys = ("top_k_vs_best_mean", "top_k_vs_best_median", "top_k_vs_best_worst",
            "shapes_within_5pct", "random_k_vs_best_mean", "default_vs_best_mean",
            "tuning_time_ratio")
    by_k = {str(kk): {key: v for key, v in evaluate(records, tuner, test_idx, k=kk).items()
                      if key in keys} for kk in (1, 2, 4)}
    # full size: the benchmark workload in both modes, and small held-out shapes
    full = [Shape(channels=1536, dms=2048, samples=24576, bits=8, subbands=0, dm_step=0.2,
                  seed=11),
            Shape(channels=1536, dms=2048, samples=24576, bits=8, subbands=32, dm_step=0.2,
                  seed=12)]
    picked = [shapes[i] for i in test_idx if direct_sum_adds(shapes[i]) <= max_full_adds]
    full += picked[:full_shapes]
    t0 = time.perf_counter()
    full_records = collect(full, device=device, full_size=True)
    t_full = time.perf_counter() - t0
    full_rep = {str(kk): evaluate(full_records, tuner, range(len(full_records)), k=kk)
                for kk in (1, 2, 4)}
    return {"k": k, "held_out": {"shapes": len(test_idx), **by_k[str(k)]},
            "by_k": by_k,
            "full_size": {"shapes": [f"{s.channels} ch x {s.dms} DM x {s.samples} samples, "
                                     f"{s.bits}-bit, {s.subbands} subbands, step {s.dm_step:.3f}"
                                     for s in full],
                          "by_k": {kk: {key: v for key, v in r.items() if key in keys}
                                   for kk, r in full_rep.items()},
                          "per_shape_top_k": full_rep[str(k)]["per_shape"],
                          "sweep_s": t_full},
            "study_shapes": count, "large_training_shapes": len(large),
            "large_collect_s": t_large,
            "train_rows": int(mask.sum()), "collect_s": t_collect,
            "train_s": t_train,
            "network": f"{members} x (3 x 128 ReLU, bf16 weights, fp32 accumulation), "
                       "trained by the library's CUDA kernels (Adam, full batch), "
                       "predictions averaged",
            "what": "held-out shapes are cut to <= 1024 DMs x 16384 samples for timing; "
                    "full_size shapes are timed whole; tuning time = building and timing the "
                    "chosen configurations plus ranking, against the same for all of them"}


# ---------------------------------------------------------------------------
# command line: the reference's DedispersionTuning switches

def registry_filter(candidates, mode: int, bits: int, a) -> list:
    """The reference tuner's limits on its enumeration
    (src/DedispersionTuning.cpp:201-283) applied to the compiled registry:
    threadsD0 from -min_threads up to -max_columns, threadsD1 up to -max_rows,
    threadsD0 x threadsD1 at most -max_threads and a multiple of -vector,
    itemsD0 up to -max_sample_items, itemsD1 up to -max_dm_items, unroll up
    to -max_unroll, and the reference's register estimate of a
    local-memory kernel, itemsD1 + itemsD0 x itemsD1 + 9 (single step) or
    + 10 (step one, two), + 4 below 8 bits, at most -max_items.  An unset
    switch (None or 0) does not filter."""
    out = []
    for k in candidates:
        c = k.conf
        t0, t1 = c.nrThreadsD0, c.nrThreadsD1
        est = c.nrItemsD1 + c.nrItemsD0 * c.nrItemsD1 + (9 if mode == DD_SINGLE_STEP else 10)
        if bits < 8:
            est += 4
        checks = (
            (getattr(a, "min_threads", None), lambda v: t0 >= v),
            (getattr(a, "max_columns", None), lambda v: t0 <= v),
            (getattr(a, "max_rows", None), lambda v: t1 <= v),
            (getattr(a, "max_threads", None), lambda v: t0 * t1 <= v),
            (getattr(a, "vector", None), lambda v: (t0 * t1) % v == 0),
            (getattr(a, "max_sample_items", None), lambda v: c.nrItemsD0 <= v),
            (getattr(a, "max_dm_items", None), lambda v: c.nrItemsD1 <= v),
            (getattr(a, "max_unroll", None), lambda v: c.unroll <= v),
            (getattr(a, "max_items", None), lambda v: est <= v),
        )
        if all(ok(v) for v, ok in checks if v):
            out.append(k)
    return out


def _args(argv):
    ap = argparse.ArgumentParser(prog="python -m dedispersion_gb300.tuning",
                                 prefix_chars="-", allow_abbrev=False)
    for flag in ("-single_step", "-step_one", "-step_two", "-best"):
        ap.add_argument(flag, action="store_true")
    for flag, typ in (("-iterations", int), ("-padding", int), ("-beams", int),
                      ("-synthesized_beams", int), ("-samples", int), ("-sampling_time", float),
                      ("-min_freq", float), ("-channel_bandwidth", float), ("-channels", int),
                      ("-subbands", int), ("-dms", int), ("-dm_first", float), ("-dm_step", float),
                      ("-subbanding_dms", int), ("-subbanding_dm_first", float),
                      ("-subbanding_dm_step", float), ("-input_bits", int),
                      ("-min_threads", int), ("-max_threads", int), ("-max_items", int),
                      ("-max_unroll", int), ("-max_rows", int), ("-max_columns", int),
                      ("-vector", int), ("-max_sample_items", int), ("-max_dm_items", int),
                      ("-opencl_platform", int), ("-opencl_device", int)):
        ap.add_argument(flag, type=typ)
    ap.add_argument("-zapped_channels")
    ap.add_argument("-device_name", default="GB300")
    ap.add_argument("-tuned_file")
    # learned tuning (no reference counterpart): rank with a saved cost model
    # and time only its top k; or train and save one
    ap.add_argument("-learned")
    ap.add_argument("-top_k", type=int, default=2)
    ap.add_argument("-train_model")
    ap.add_argument("-study_shapes", type=int, default=400)
    return ap.parse_args(argv)


def main(argv=None) -> int:
    a = _args(argv if argv is not None else sys.argv[1:])
    if a.train_model:
        print(json.dumps(train_model(a.train_model, count=a.study_shapes)))
        return 0
    if a.single_step + a.step_one + a.step_two != 1:
        print("Mutually exclusive modes, select one: -single_step -step_one -step_two",
              file=sys.stderr)
        return 1
    from . import Observation
    o = Observation()
    o.setNrBeams(a.beams or 1)
    o.setNrSamplesPerBatch(a.samples)
    o.setSamplingTime(a.sampling_time)
    bits = a.input_bits or 8
    if a.single_step:
        o.setNrSynthesizedBeams(a.synthesized_beams or 1)
        o.setFrequencyRange(1, a.channels, a.min_freq, a.channel_bandwidth)
        o.setDMRange(a.dms, a.dm_first, a.dm_step)
        mode = DD_SINGLE_STEP
    else:
        o.setNrSynthesizedBeams(a.synthesized_beams or 1)
        o.setFrequencyRange(a.subbands, a.channels, a.min_freq, a.channel_bandwidth)
        o.setDMRange(a.subbanding_dms, a.subbanding_dm_first or 0.0, a.subbanding_dm_step or 0.0,
                     True)
        o.setDMRange(a.dms, a.dm_first, a.dm_step)
        mode = DD_STEP_ONE if a.step_one else DD_STEP_TWO
    padding = a.padding
    shifts = getShifts(o, padding)
    from . import getShiftsStepTwo
    shifts2 = getShiftsStepTwo(o, padding) if not a.single_step else None
    zapped = np.zeros(o.getNrChannels(padding // 4), np.uint32)
    if a.zapped_channels:
        for tok in open(a.zapped_channels).read().split():
            c = int(tok)
            if 0 <= c < o.getNrChannels():
                zapped[c] = 1
    # dispersed lengths as DedispersionTuning sets them (src/DedispersionTuning.cpp:131-143)
    if a.single_step:
        o.setNrSamplesPerDispersedBatch(syn.dispersed_samples(a.samples, shifts[0], a.dm_first,
                                                              a.dms, a.dm_step))
    else:
        s1 = syn.dispersed_samples(a.samples, shifts2[0], a.dm_first, a.dms, a.dm_step)
        o.setNrSamplesPerBatch(s1, True)
        o.setNrSamplesPerDispersedBatch(syn.dispersed_samples(
            s1, shifts[0], a.subbanding_dm_first or 0.0, a.subbanding_dms,
            a.subbanding_dm_step or 0.0), True)
    cands = registry_filter(family_kernels(mode, bits), mode, bits, a)
    if a.learned and not a.step_two:
        # time only the cost model's top k (step two has no model: full sweep)
        tuner = LearnedTuner.load(a.learned)
        n = len(cands)
        cands = tuner.rank(observation_shape(o, mode, bits, shifts), cands)[:max(1, a.top_k)]
        print(f"learned: timed {len(cands)} of {n} configurations", file=sys.stderr)
    res = sweep(o, mode, bits, padding, shifts2 if a.step_two else shifts,
                zapped if not a.step_two else None, None, iterations=a.iterations or 3,
                candidates=cands)
    if a.best:
        best = res[0]
        line = f"{a.dms if not a.step_one else a.subbanding_dms} {best.conf.print()}"
        print(line)
        if a.tuned_file:
            from . import writeTunedDedispersionConf
            writeTunedDedispersionConf(a.tuned_file, a.device_name,
                                       a.dms if not a.step_one else a.subbanding_dms, best.conf)
        return 0
    print("# nrBeams nrSynthesizedBeams nrSubbandingDMs nrDMs nrSubbands nrChannels "
          "nrZappedChannels nrSamplesSubbanding nrSamples *configuration* GFLOP/s time "
          "stdDeviation COV\n")
    nz = int(zapped[:o.getNrChannels()].sum())
    for r in res:
        cov = r.std_ms / r.mean_ms if r.mean_ms else 0.0
        print(f"{o.getNrBeams()} {o.getNrSynthesizedBeams()} {o.getNrDMs(True)} {o.getNrDMs()} "
              f"{o.getNrSubbands()} {o.getNrChannels()} {nz} {o.getNrSamplesPerBatch(True)} "
              f"{o.getNrSamplesPerBatch()} {r.conf.print()} {r.gflops:.3f} "
              f"{r.mean_ms * 1e-3:.6f} {r.std_ms * 1e-3:.6f} {cov:.6f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
