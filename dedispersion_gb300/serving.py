"""Real-time serving of many beams of batch streams.

Each beam is a ``dd_stream`` (dedispersion_gb300/csrc/dd_stream.cu): device
ring rows [max-delay tail | new batch], a pinned staging input and a pinned
output, and one recorded CUDA graph per push (copy in, dedisperse -- single
step, or step one then step two --, copy out, carry the tail).  The server:

* admits beams against an HBM budget, from each stream's device bytes known
  before it is created (``dd_stream_bytes``); a beam that does not fit is
  refused with DD_ERR_OVER_BUDGET;
* runs a schedule of batch arrivals (per beam a batch every period, delayed
  by an exponential jitter -- Poisson-jittered arrivals), one CUDA stream per
  beam so that beams overlap on the GPU, one batch in flight per staging
  buffer of a beam (two when double-buffered) and later arrivals of a busy
  beam queued; the beams' host staging copies run on a pool of threads;
* injects host-side faults on request (:func:`inject`): late batches and
  batches whose data never arrive (pushed as zeros, counted as dropped);
* reports per-batch latency (arrival -> output in host memory), p50/p99
  against the deadline (the batch period), and throughput in DM-samples/s.

No counterpart in the reference: its streaming mode (splitBatches) was never
implemented (include/Dedispersion.hpp:202; README.md:76-79).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import (DedispersionError, Observation, _abi, getShifts, getShiftsStepTwo)
from ._abi import check, lib
from . import synthetic as syn


@dataclass
class BeamConfig:
    """One beam's stream: 2.048 s batches of 25000 samples at 81.92 us by default."""

    name: str = "beam"
    channels: int = 1536
    min_freq: float = 1220.0
    bandwidth: float = 0.1953125
    sampling_time: float = 81.92e-6
    samples: int = 25000
    dms: int = 2048
    dm_step: float = 0.2
    first_dm: float = 0.0
    bits: int = 8
    subband: bool = False
    subbands: int = 32
    dms_per_subband_dm: int = 32   # step-two DMs per step-one DM (subband mode)
    padding: int = 128
    zap_fraction: float = 0.05
    seed: int = 0
    double_buffer: bool = False    # two pinned staging/output pairs, two batches in flight
    time_major: bool = False       # batches arrive as file-order [samples][channels] blocks
    reverse: bool = False          # (time-major) file channel 0 is the highest frequency

    @property
    def period(self) -> float:
        return self.samples * self.sampling_time

    def observation(self) -> Observation:
        o = Observation()
        o.setNrBeams(1)
        o.setNrSynthesizedBeams(1)
        o.setNrSamplesPerBatch(self.samples)
        o.setSamplingTime(self.sampling_time)
        if self.subband:
            o.setFrequencyRange(self.subbands, self.channels, self.min_freq, self.bandwidth)
            d2 = self.dms_per_subband_dm
            if self.dms % d2:
                raise ValueError("dms must be a multiple of dms_per_subband_dm")
            o.setDMRange(self.dms // d2, self.first_dm, self.dm_step * d2, True)
            o.setDMRange(d2, 0.0, self.dm_step)
        else:
            o.setFrequencyRange(1, self.channels, self.min_freq, self.bandwidth)
            o.setDMRange(self.dms, self.first_dm, self.dm_step)
        return o

    def tables(self):
        obs = self.observation()
        shifts = getShifts(obs, self.padding)
        shifts2 = getShiftsStepTwo(obs, self.padding) if self.subband else None
        zapped = syn.zapped_mask(self.channels, self.zap_fraction, self.seed, self.padding)
        return obs, shifts, shifts2, zapped


def _f32p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def stream_bytes(cfg: BeamConfig) -> tuple[int, int]:
    """(device bytes, carried tail samples) of a beam's stream, without a device."""
    obs, shifts, shifts2, zapped = cfg.tables()
    nbytes, tail = C.c_uint64(0), C.c_uint32(0)
    check(lib().dd_stream_bytes(C.byref(obs.c), int(cfg.subband), cfg.bits, cfg.padding,
                                _f32p(shifts), _f32p(shifts2),
                                zapped.ctypes.data_as(C.POINTER(C.c_uint32)),
                                C.byref(nbytes), C.byref(tail)))
    return nbytes.value, tail.value


class Stream:
    """One beam's device stream (wraps dd_stream)."""

    def __init__(self, cfg: BeamConfig, device: int = 0):
        self.cfg = cfg
        self.obs, self.shifts, self.shifts2, self.zapped = cfg.tables()
        self._h = C.c_void_p()
        check(lib().dd_stream_create(C.byref(self._h), C.byref(self.obs.c), int(cfg.subband),
                                     cfg.bits, cfg.padding, _f32p(self.shifts),
                                     _f32p(self.shifts2),
                                     self.zapped.ctypes.data_as(C.POINTER(C.c_uint32)), device))
        tail, nbytes = C.c_uint32(0), C.c_uint64(0)
        row, rows = C.c_uint64(0), C.c_uint32(0)
        check(lib().dd_stream_info(self._h, C.byref(tail), C.byref(nbytes), C.byref(row),
                                   C.byref(rows)))
        self.tail, self.device_bytes = tail.value, nbytes.value
        self.input_row_bytes, self.output_rows = row.value, rows.value
        self.nbuf, self.time_major = 1, False
        self._map_buffers()
        self.output = self.outputs[0]
        self.dm_samples = self.output_rows * self.cfg.samples

    def _map_buffers(self) -> None:
        """numpy views of every pinned staging/output pair."""
        cfg = self.cfg
        self.stagings, self.outputs = [], []
        for i in range(self.nbuf):
            h_in, h_out = C.c_void_p(), C.c_void_p()
            check(lib().dd_stream_buffer(self._h, i, C.byref(h_in), C.byref(h_out)))
            n_in = cfg.channels * self.input_row_bytes
            st = np.ctypeslib.as_array(C.cast(h_in, C.POINTER(C.c_uint8)), shape=(n_in,))
            st = (st[:cfg.samples * cfg.channels].reshape(cfg.samples, cfg.channels)
                  if self.time_major else st.reshape(cfg.channels, -1))
            self.stagings.append(st)
            self.outputs.append(np.ctypeslib.as_array(
                C.cast(h_out, C.POINTER(C.c_float)),
                shape=(self.output_rows * cfg.samples,)).reshape(self.output_rows, cfg.samples))

    @property
    def next_buffer(self) -> int:
        i = C.c_int(0)
        check(lib().dd_stream_next_buffer(self._h, C.byref(i)))
        return i.value

    @property
    def staging(self) -> np.ndarray:
        """The staging input the next push reads."""
        return self.stagings[self.next_buffer]

    def set_double_buffer(self, enable: bool = True) -> None:
        """Two staging/output pairs used in turn: the next batch can be
        staged while a push is in flight (dd_stream_set_double_buffer)."""
        check(lib().dd_stream_set_double_buffer(self._h, 1 if enable else 0))
        self.nbuf = 2 if enable else 1
        self._map_buffers()

    def set_time_major(self, reverse: bool = False) -> None:
        """Take batches as time-major 8-bit blocks (file order); ``staging``
        becomes a [samples][channels] view of the same pinned buffer."""
        check(lib().dd_stream_set_time_major(self._h, 1 if reverse else 0))
        self.time_major = True
        self._map_buffers()
        tail, nbytes = C.c_uint32(0), C.c_uint64(0)
        check(lib().dd_stream_info(self._h, C.byref(tail), C.byref(nbytes), None, None))
        self.device_bytes = nbytes.value

    def push(self, cuda_stream) -> int:
        """Enqueue the staged batch; returns the buffer pair it uses (its
        output lands in ``outputs[index]``, also ``output``)."""
        s = cuda_stream if isinstance(cuda_stream, int) else int(cuda_stream.cuda_stream)
        index = self.next_buffer
        check(lib().dd_stream_push(self._h, C.c_void_p(s)))
        self.output = self.outputs[index]
        return index

    def close(self) -> None:
        if self._h:
            lib().dd_stream_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def served_beams(count: int = 12, seed: int = 77, padding: int = 128,
                 double_buffer: bool = True) -> list[BeamConfig]:
    """The 12-beam real-time workload: 2.048 s batches (1536 channels, 25000
    samples at 81.92 us, 8-bit), each beam's DM count drawn uniformly from
    1024-4096 in steps of 128 at step 0.2, even beams single step and odd
    beams 32-subband, 5 % of channels zapped from the beam's seed."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(count):
        dms = int(rng.integers(8, 33)) * 128
        out.append(BeamConfig(name=f"beam{b}", dms=dms, subband=(b % 2 == 1), seed=100 + b,
                              padding=padding, double_buffer=double_buffer))
    return out


class FileSource:
    """A `source` for Server.serve that reads each beam's batches straight
    from its SIGPROC filterbank or PSRDADA file (``ingest.Filterbank`` /
    ``ingest.Dada``, 8-bit) into the stream's pinned staging: batch k of beam
    b is samples [k S, (k + 1) S) of its file, past the end zeros.  The
    beams are admitted with ``time_major`` (and ``reverse`` = the file's
    channel order), so the file-order block goes to the device as it is and
    is transposed into the ring there.  With the server's staging pool and
    double-buffered streams, a beam's next read overlaps the GPU work of its
    batch in flight: file -> pinned host -> device ring, no other host copy."""

    def __init__(self, files) -> None:
        self.files = list(files)

    @staticmethod
    def config(file, name: str, **kw) -> BeamConfig:
        """A BeamConfig matching a file's channels, band and sampling time."""
        obs = file.observation(Observation())
        return BeamConfig(name=name, channels=obs.getNrChannels(), min_freq=obs.getMinFreq(),
                          bandwidth=obs.getChannelBandwidth(),
                          sampling_time=obs.getSamplingTime(), time_major=True,
                          reverse=file.reversed, **kw)

    def __call__(self, b: int, k: int, staging: np.ndarray) -> None:
        self.files[b].read_into(k * staging.shape[0], staging)


def poisson_schedule(beams: int, batches: int, period: float, jitter: float, seed: int):
    """Arrivals (time, beam, batch): batch k of beam b at phase_b + k * period +
    Exp(jitter), sorted by time."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(beams):
        phase = float(rng.uniform(0.0, period))
        for k in range(batches):
            out.append((phase + k * period + float(rng.exponential(jitter)), b, k))
    out.sort()
    return out


# Marks a scheduled batch whose data never arrived (see Server.serve).
DROPPED = "dropped"


def inject(schedule, late: dict | None = None, dropped=()):
    """A copy of `schedule` [(arrival s, beam, batch)] with faults injected on
    the host: ``late`` maps (beam, batch) to a delay in seconds added to that
    batch's arrival; ``dropped`` lists (beam, batch) pairs whose data never
    arrive.  Entries become (nominal arrival, beam, batch, delay or DROPPED)."""
    late = late or {}
    dropped = set(dropped)
    out = []
    for t, b, k in (e[:3] for e in schedule):
        if (b, k) in dropped:
            out.append((t, b, k, DROPPED))
        else:
            out.append((t, b, k, float(late.get((b, k), 0.0))))
    return out


@dataclass
class ServeReport:
    latencies: list = field(default_factory=list)  # seconds, per delivered batch
    misses: list = field(default_factory=list)     # (beam, batch) past their deadline
    dropped: list = field(default_factory=list)    # (beam, batch) whose data never came
    late: list = field(default_factory=list)       # (beam, batch) that arrived late
    dm_samples: int = 0
    wall: float = 0.0
    deadline: float = 0.0
    time_compression: float = 1.0

    def summary(self) -> dict:
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return {"batches": len(self.latencies),
                "p50_latency_s": float(np.percentile(lat, 50)),
                "p99_latency_s": float(np.percentile(lat, 99)),
                "max_latency_s": float(lat.max()),
                "deadline_s": self.deadline,
                "deadline_misses": len(self.misses),
                "dropped_batches": len(self.dropped),
                "late_batches": len(self.late),
                "throughput_dm_samples_per_s": self.dm_samples / self.wall if self.wall else 0.0,
                "wall_s": self.wall, "time_compression": self.time_compression}


class Server:
    """Admits beams against an HBM budget and serves their batch streams."""

    def __init__(self, budget_bytes: int = 150 * 10**9, device: int = 0):
        self.budget = int(budget_bytes)
        self.device = device
        self.used = 0
        self.streams: list[Stream] = []

    def admit(self, cfg: BeamConfig) -> Stream:
        need, _ = stream_bytes(cfg)
        if cfg.time_major:
            need += cfg.samples * cfg.channels  # the device block transposed into the ring
        if self.used + need > self.budget:
            raise DedispersionError(_abi.DD_ERR_OVER_BUDGET,
                                    f"beam {cfg.name} needs {need} device bytes, "
                                    f"{self.budget - self.used} of the budget are left")
        s = Stream(cfg, self.device)
        if cfg.time_major:
            s.set_time_major(cfg.reverse)
        if cfg.double_buffer:
            s.set_double_buffer(True)
        self.used += s.device_bytes
        self.streams.append(s)
        return s

    def close(self) -> None:
        for s in self.streams:
            s.close()
        self.streams.clear()
        self.used = 0

    def serve(self, schedule, source, consumer=None, time_compression: float = 1.0,
              deadline: float | None = None, workers: int | None = None) -> ServeReport:
        """Run `schedule`: entries (arrival s, beam, batch), or (nominal
        arrival s, beam, batch, delay s or DROPPED) as :func:`inject` makes
        them.  source(beam, batch, staging) fills a beam's pinned staging
        input; consumer(beam, batch, output) sees each finished output
        (pinned host rows).

        A beam's batches are pushed in batch order, whatever order they
        arrive in: the device ring carries each batch's tail into the next.
        A late batch (delay > 0) arrives `delay` after its nominal time; its
        later batches wait for it.  A dropped batch is pushed as zeros, so
        that the ring stays aligned in time, and is neither delivered nor
        timed.  Latency runs from a batch's actual arrival to its output on
        the host; a batch misses its deadline when its output lands more
        than `deadline` (default: the longest batch period) after its
        nominal arrival.

        Staging a batch (the source's copy into pinned memory) and its push
        run on a pool of `workers` host threads (default: one per beam, at
        most 8), one batch of a beam at a time, so that the beams' host
        copies overlap each other and the GPU's work, as the beams' receiver
        threads would in a telescope's pipeline."""
        import os
        from concurrent.futures import ThreadPoolExecutor

        import torch
        n = len(self.streams)
        if workers is None:
            workers = max(1, min(n, 8, os.cpu_count() or 1))
        cuda_streams = [torch.cuda.Stream(device=self.device) for _ in range(n)]
        arrivals = []
        for e in schedule:
            t, b, k = e[:3]
            extra = e[3] if len(e) > 3 else 0.0
            drop = extra == DROPPED
            arrivals.append((t if drop else t + float(extra), b, k, t, drop))
        arrivals.sort(key=lambda a: a[0])
        next_k = [None] * n                  # the batch each beam pushes next
        for _, b, k, _, _ in arrivals:
            next_k[b] = k if next_k[b] is None else min(next_k[b], k)
        pending = [{} for _ in range(n)]     # arrived: batch -> (t actual, t nominal, dropped)
        # in flight on the GPU, oldest first: (event, batch, buffer, t actual,
        # t nominal, dropped); up to one per staging buffer of the beam's stream
        inflight = [[] for _ in range(n)]
        staging = [None] * n                 # the beam's batch being staged: (future, ...)
        report = ServeReport(deadline=deadline if deadline is not None
                             else max(s.cfg.period for s in self.streams),
                             time_compression=time_compression)
        device = self.device

        def stage_and_push(b, k, drop):
            torch.cuda.set_device(device)
            st = self.streams[b]
            if drop:
                st.staging[...] = 0
            else:
                source(b, k, st.staging)
            idx = st.push(cuda_streams[b])
            ev = torch.cuda.Event()
            ev.record(cuda_streams[b])
            return ev, idx

        pool = ThreadPoolExecutor(max_workers=workers)
        t0 = time.perf_counter()

        def now():
            return (time.perf_counter() - t0) * time_compression

        def finish(b):
            ev, k, idx, ta, tn, drop = inflight[b].pop(0)
            done = now()
            if drop:
                report.dropped.append((b, k))
                return
            report.latencies.append((done - ta) / time_compression)
            if done - tn > report.deadline * time_compression:
                report.misses.append((b, k))
            report.dm_samples += self.streams[b].dm_samples
            if consumer is not None:
                consumer(b, k, self.streams[b].outputs[idx])

        def dispatch(b):
            if staging[b] is not None:
                fut, k, ta, tn, drop = staging[b]
                if not fut.done():
                    return
                ev, idx = fut.result()
                inflight[b].append((ev, k, idx, ta, tn, drop))
                staging[b] = None
            st = self.streams[b]
            if next_k[b] in pending[b] and len(inflight[b]) < st.nbuf:
                k = next_k[b]
                ta, tn, drop = pending[b].pop(k)
                staging[b] = (pool.submit(stage_and_push, b, k, drop), k, ta, tn, drop)
                next_k[b] = k + 1

        def poll():
            for b in range(n):
                while inflight[b] and inflight[b][0][0].query():
                    finish(b)
                dispatch(b)

        try:
            for ta, b, k, tn, drop in arrivals:
                while now() < ta:
                    poll()
                    time.sleep(0.0002)
                if ta > tn:
                    report.late.append((b, k))
                pending[b][k] = (ta, tn, drop)
                poll()
            while any(inflight) or any(pending) or any(x is not None for x in staging):
                if (not any(inflight) and all(x is None for x in staging) and
                        all(next_k[b] not in pending[b] for b in range(n) if pending[b])):
                    raise ValueError("schedule has a gap: batches "
                                     f"{[(b, sorted(p)) for b, p in enumerate(pending) if p]} "
                                     "wait for batches that never arrive")
                poll()
                time.sleep(0.0002)
        finally:
            pool.shutdown(wait=True)
        report.wall = (time.perf_counter() - t0)
        return report
