"""Throughput benchmark of the dedispersion engine on the 1536-channel,
2048-DM, 24576-sample 8-bit workload (single step, bit-exact integer sums).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Metric: DM-samples/s = DM trials x output
samples per second.

* value      -- device-resident: K back-to-back runs of the plain kernel on
                inputs already in HBM, timed with CUDA events on the launching
                stream.  Inputs rotate over 4 buffers (4 x 45 MB) while every
                step also writes its 201 MB output, so each step starts with its
                input out of L2.
* e2e        -- the same metric through the C ABI's synchronous host-buffer
                call dd_dedispersion (the reference's drop-in): pinned host
                input copied to the device, kernel, output copied back, all
                inside the timed region.
* roofline   -- the path is add-bound (1459 live channels: 1459 adds per
                DM-sample of the direct sum against 4.9 compulsory bytes);
                achieved = direct-sum adds / launch time over the scalar add
                rate of 152 SMs x 128 lanes at the SM clock sampled during the
                run.  The default kernel reaches the same integer sums with
                fewer adds (partial sums shared by DMs with equal relative
                delays); `executed` reports the adds it performs.  The HBM view
                of the same launch is included.
* cpu_baseline -- the CPU oracle (a loop-for-loop port of the reference's
                dedispersion) on all host cores over a DM prefix of the same
                workload.

With --impl reference the CPU port alone is timed, each step a DM prefix of
the workload, on all host threads.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DM-samples/s (DM trials x output samples per second), 1536ch x 2048DM x 24576 8-bit, bit-exact"
UNIT = "DM-samples/s"
WORKLOAD = "single-step 1536ch x 2048DM x 24576 samples, uint8 N(128,20) + 20 pulses, 5% zapped"
PADDING = 128
SMS = 152
LANES = 128


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=2.0,
                    help="target wall time of the CPU baseline sample")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 40-beam batched measurement")
    ap.add_argument("--no-served", action="store_true",
                    help="skip the 12-beam serving measurement")
    ap.add_argument("--served-only", action="store_true",
                    help="run only the 12-beam serving measurement and print its object")
    ap.add_argument("--no-tuning", action="store_true",
                    help="skip the learned-tuner measurement (400-shape sweep and training)")
    ap.add_argument("--kernel", default=None,
                    help="registry name of the tile configuration to run (default: the "
                         "library's default for the workload)")
    ap.add_argument("--kernel-only", action="store_true",
                    help="run only the warm-up and timed kernel launches (the command ncu "
                         "captures); prints the device-resident figure alone")
    ap.add_argument("--float-only", action="store_true",
                    help="run only the float32-input line (--steps runs after 2 warm-up runs; "
                         "the command ncu captures for the float kernel)")
    ap.add_argument("--float-dms", type=int, default=None, metavar="D",
                    help="with --float-only: the first D of the 2048 DM trials (a smaller case "
                         "of the same rows for a full ncu capture)")
    ap.add_argument("--float-kernel", default=None,
                    help="registry name of the float tile for the float32 line (default: the "
                         "library's float default)")
    ap.add_argument("--subband-only", type=int, default=None, metavar="CHUNKS",
                    help="run only the subband pipeline, --warmup + --steps runs with "
                         "dd_subband_set_chunks(CHUNKS) (the command ncu captures for the "
                         "intermediate's DRAM traffic); prints its time per batch")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def beam_seed(rank):
    """Each rank dedisperses its own beam (weak scaling): beams are independent,
    so ranks share no data and no collective sits on the data path."""
    return 1 + rank


def max_over_ranks(seconds, pg, device):
    """The job's elapsed time: the slowest rank's (all_reduce MAX)."""
    if pg is None:
        return seconds
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_value(world, steps, dms, samples, seconds):
    """Whole-job DM-samples/s: every rank's units over the slowest rank's time."""
    return world * steps * dms * samples / seconds


def workload(seed=1):
    import dedispersion_gb300 as dd
    from dedispersion_gb300 import synthetic as syn
    obs = syn.large_observation(PADDING)
    shifts = dd.getShifts(obs, PADDING)
    zapped = syn.zapped_mask(1536, 0.05, 7, PADDING)
    mapping = syn.identity_mapping(obs, PADDING)
    inp = syn.make_input(obs, 8, PADDING, seed=seed, mean=128.0, sigma=20.0, pulses=20,
                         shifts=shifts)
    return obs, shifts, zapped, mapping, inp


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]),
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def read_profile_traffic():
    """DRAM bytes per launch of the plain kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "shared8_plain_1536ch_2048dm_8bit.md"
    if not p.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9]+)", p.read_text())
    return int(m.group(1)) if m else None


def cpu_sample(o, sh, z, m, inp, target_s, threads):
    """Time the oracle port on a DM prefix of the single-step workload sized
    for ~target_s of wall time; returns (DM-samples/s, dms, seconds).  The
    prefix keeps the first DM, the DM step and the full dispersed length, so
    every delay is the full workload's.  ``o`` is the observation struct
    (oracle.types or the engine's, same layout)."""
    import oracle
    out = np.zeros(o.nr_dms * out_row(o), dtype=np.float32)
    dms = 2
    while True:
        t = time.perf_counter()
        oracle.dedispersion(o, z, m, inp, out, sh, PADDING, 8, 0, dms, threads)
        dt = time.perf_counter() - t
        if dt >= target_s * 0.5 or dms >= o.nr_dms:
            return dms * o.nr_samples_per_batch / dt, dms, dt
        dms = min(o.nr_dms, max(dms + 1, int(dms * target_s / max(dt, 1e-3))))


def reference_cpu_sample(o, sh, z, m, inp, target_s):
    """The reference's own CPU template (include/Dedispersion.hpp:70-109,
    compiled unmodified into oracle/_ref/libddref.so), single-threaded as the
    reference runs it, on a DM prefix sized for ~target_s.  None where that
    library was not built (the reference's sources are not on this machine).
    Returns (DM-samples/s, dms, seconds)."""
    import ctypes as C
    import oracle
    if not oracle.REF_LIB.exists():
        return None
    ref = oracle.reference()
    U32P, F32P = C.POINTER(C.c_uint32), C.POINTER(C.c_float)
    dms = 1
    while True:
        sub = type(o).from_buffer_copy(o)
        sub.nr_dms = dms          # same first DM, step and dispersed length
        out = np.zeros(dms * out_row(o), dtype=np.float32)
        t = time.perf_counter()
        rc = ref.ddref_dedispersion(C.byref(sub), z.ctypes.data_as(U32P), z.size,
                                    m.ctypes.data_as(U32P), m.size,
                                    C.c_void_p(inp.ctypes.data), inp.size,
                                    out.ctypes.data_as(F32P), out.size,
                                    sh.ctypes.data_as(F32P), sh.size, PADDING, 8)
        dt = time.perf_counter() - t
        if rc != 0:
            return None
        if dt >= target_s * 0.5 or dms >= o.nr_dms:
            return dms * o.nr_samples_per_batch / dt, dms, dt
        dms = min(o.nr_dms, max(dms + 1, int(dms * target_s / max(dt, 1e-3))))


def cpu_baseline(o, sh, z, m, inp, target_s):
    """cpu_baseline object: the oracle port on every host thread (the figure),
    the same port on one thread, and the reference's own code on one thread
    where it was built here."""
    threads = os.cpu_count() or 1
    val, dms, dt = cpu_sample(o, sh, z, m, inp, target_s, threads)
    one, dms1, dt1 = cpu_sample(o, sh, z, m, inp, target_s / 2, 1)
    line = {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"DMs 0..{dms - 1} of 2048 (all 24576 samples, 1536 channels), "
                      f"{dt:.2f} s wall on {threads} threads",
            "single_thread": {"value": one, "cores": 1, "kind": "port",
                              "sample": f"DMs 0..{dms1 - 1}, {dt1:.2f} s on 1 thread"}}
    ref = reference_cpu_sample(o, sh, z, m, inp, target_s / 2)
    if ref is None:
        line["reference_code"] = ("not run: the reference's sources are not on this machine, "
                                  "so oracle/_ref was not built; the port is bit-identical to it "
                                  "(tests/test_oracle.py)")
    else:
        line["reference_code"] = {"value": ref[0], "cores": 1, "kind": "reference",
                                  "sample": f"DMs 0..{ref[1] - 1}, {ref[2]:.2f} s on 1 thread"}
    return line


def out_row(o):
    """Padded output row of the single-step layout, in floats."""
    q = PADDING // 4
    return -(-o.nr_samples_per_batch // q) * q


def bench_detect(torch, plan, d_in, d_out, stream, D, S, steps):
    """The same launches with per-DM detection statistics (sum, sum of squares,
    peak) accumulated in the same pass; reports its cost over the plain run and
    the best S/N row of the last step."""
    import dedispersion_gb300 as dd
    d_acc = torch.empty((D, 3), dtype=torch.int64, device=d_out.device)
    n = max(3, min(steps, 20))
    plan.setOverlap(False)  # both sides launched one after another
    for i in range(3):
        plan.run_stats(d_in[i % len(d_in)], d_out, d_acc, stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for i in range(n):
        plan.run(d_in[i % len(d_in)], d_out, stream)
    e1.record(stream)
    for i in range(n):
        plan.run_stats(d_in[i % len(d_in)], d_out, d_acc, stream)
    e2.record(stream)
    plan.check(stream)
    plan.setOverlap(True)
    plain_ms, stats_ms = e0.elapsed_time(e1) / n, e1.elapsed_time(e2) / n
    st = dd.dm_stats(d_acc.cpu().numpy().view(np.uint64), S)
    best = int(np.argmax(st["snr"]))
    return {"ms_per_step": stats_ms, "plain_ms_per_step": plain_ms,
            "overhead": stats_ms / plain_ms - 1.0,
            "fused_in_kernel": plan.conf().getNrItemsD2() == 8,
            "best_row": {"dm_index": best, "snr": float(st["snr"][best]),
                         "peak_sample": int(st["peak_sample"][best])},
            "what": "per-DM sum, sum of squares and earliest peak of the output, exact "
                    "integers, accumulated while dedispersing (dd_plan_run_stats)"}


def bench_ingest(torch, inp, lay, obs, stream):
    """Filterbank samples arrive time-major ([sample][channel]); the device
    transpose puts this workload's whole input (29568 samples x 1536
    channels, 45 MB) into channel rows.  Bytes moved = read + write."""
    import ctypes as C
    from dedispersion_gb300._abi import check, lib
    S_disp, nch = obs.getNrSamplesPerDispersedBatch(), obs.getNrChannels()
    rows = inp.reshape(nch, lay.input_row_bytes)[:, :S_disp]
    d_src = torch.from_numpy(np.ascontiguousarray(rows[::-1].T)).cuda()
    d_dst = torch.zeros(lay.input_bytes, dtype=torch.uint8, device=d_src.device)
    n = 20

    def once():
        check(lib().dd_transpose_time_major(C.c_void_p(d_src.data_ptr()), S_disp, nch, 1,
                                            C.c_void_p(d_dst.data_ptr()), lay.input_row_bytes,
                                            0, C.c_void_p(stream.cuda_stream)))
    for _ in range(3):
        once()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(n):
        once()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    exact = bool(np.array_equal(d_dst.cpu().numpy().reshape(nch, -1)[:, :S_disp], rows))
    moved = 2 * S_disp * nch
    try:
        peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"]
    except Exception:
        peak = 6784.2
    return {"ms": ms, "gbs": moved / ms / 1e6, "hbm_frac": moved / ms / 1e6 / peak,
            "bytes": moved, "exact": exact,
            "what": "time-major filterbank block -> channel rows (dd_transpose_time_major), "
                    "descending-frequency file order reversed on the way"}


def bench_float(torch, device: int, steps: int, peak_adds: float, kernel: str | None = None,
                dms: int | None = None):
    """Config 2 with float32 input (N(128, 20), same channels, DMs, zapping):
    throughput of the float path (summed in the reference's channel order),
    and its largest relative error against an FP64 sum of four DM rows
    computed here with numpy.  `dms` keeps only the first DM trials (the
    profiling case)."""
    import dedispersion_gb300 as dd
    from dedispersion_gb300 import synthetic as syn
    obs = syn.large_observation(PADDING)
    if dms:
        obs.setDMRange(dms, obs.getFirstDM(), obs.getDMStep())
    shifts = dd.getShifts(obs, PADDING)
    zapped = syn.zapped_mask(1536, 0.05, 7, PADDING)
    mapping = syn.identity_mapping(obs, PADDING)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 32, PADDING)
    C, S, D = 1536, obs.getNrSamplesPerBatch(), obs.getNrDMs()
    row = lay.input_row_bytes // 4
    n = obs.getNrSamplesPerDispersedBatch()
    g = torch.Generator(device=f"cuda:{device}")
    g.manual_seed(5)
    d_in = torch.zeros((C, row), dtype=torch.float32, device=f"cuda:{device}")
    d_in[:, :n] = torch.randn((C, n), generator=g, device=f"cuda:{device}") * 20.0 + 128.0
    d_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32, device=f"cuda:{device}")
    kidx = None
    if kernel:
        kidx = next((k.index for k in dd.kernels() if k.name == kernel), None)
        if kidx is None:
            raise SystemExit(f"no compiled configuration named {kernel}")
    p = dd.Plan(obs, dd.DD_SINGLE_STEP, 32, PADDING, device=device, kernel=kidx)
    p.setShifts(shifts)
    p.setZappedChannels(zapped)
    p.setBeamMapping(mapping)
    stream = torch.cuda.current_stream()
    for _ in range(2):
        p.run(d_in, d_out, stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        p.run(d_in, d_out, stream)
    e1.record(stream)
    p.check(stream)
    t = e0.elapsed_time(e1) / 1e3 / steps
    # FP64 reference of four DM rows (0, D/3, 2D/3, D-1; float32 delay arithmetic)
    host = d_in.cpu().numpy().astype(np.float64)
    out = d_out.cpu().numpy().reshape(D, -1)[:, :S]
    live = np.flatnonzero(zapped[:C] == 0)
    err = 0.0
    for d in sorted({0, D // 3, 2 * D // 3, D - 1}):
        dm = np.float32(obs.getFirstDM()) + np.float32(d) * np.float32(obs.getDMStep())
        delay = (np.float32(dm) * shifts[live].astype(np.float32)).astype(np.uint32)
        ref = np.zeros(S, np.float64)
        for c, dl in zip(live, delay):
            ref += host[c, dl:dl + S]
        err = max(err, float(np.max(np.abs(out[d] - ref) / np.abs(ref))))
    kernel = next((k.name for k in dd.kernels()
                   if k.elem_bits == 32 and k.conf.print() == p.conf().print()), "?")
    p.close()
    adds = D * S * len(live)
    return {"value": D * S / t, "unit": UNIT, "ms_per_step": t * 1e3, "dtype": "f32",
            "adds_frac": adds / t / peak_adds, "max_rel_err_vs_fp64": err,
            "tolerance": 1e-5, "kernel": kernel,
            "workload": "1536 ch x 2048 DM x 24576 samples, float32 N(128, 20), 5% zapped"}


def subband_inputs(torch, device: int):
    """The subband workload's pipeline and device buffers (4 rotating inputs)."""
    import dedispersion_gb300 as dd
    from dedispersion_gb300 import synthetic as syn
    obs = syn.large_observation(PADDING, subbands=True)
    sh1, sh2 = dd.getShifts(obs, PADDING), dd.getShiftsStepTwo(obs, PADDING)
    zapped = syn.zapped_mask(1536, 0.05, 7, PADDING)
    mapping = syn.identity_mapping(obs, PADDING, subbands=True)
    inp = syn.make_input(obs, 8, PADDING, seed=3, mode=dd.DD_STEP_ONE, mean=128.0, sigma=20.0)
    l2 = dd.layout(obs, dd.DD_STEP_TWO, 32, PADDING)
    dev = f"cuda:{device}"
    d_in = [torch.from_numpy(inp).to(dev) for _ in range(4)]
    out = torch.empty(l2.output_bytes // 4, dtype=torch.float32, device=dev)
    pipe = dd.SubbandPipeline(obs, 8, PADDING, device=device)
    pipe.setTables(sh1, sh2, zapped, mapping)
    return obs, sh1, sh2, zapped, mapping, d_in, out, pipe


def subband_only(torch, device: int, chunks: int, steps: int, warmup: int):
    """--subband-only: the pipeline alone with `chunks` time ranges."""
    obs, _, _, _, _, d_in, out, pipe = subband_inputs(torch, device)
    pipe.setChunks(chunks)
    stream = torch.cuda.current_stream()
    for i in range(warmup):
        pipe.run(d_in[i % 4], out, stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        pipe.run(d_in[i % 4], out, stream)
    e1.record(stream)
    pipe.check(stream)
    ms = e0.elapsed_time(e1) / max(steps, 1)
    pipe.close()
    return {"subband_only": True, "chunks": chunks, "steps": steps, "ms_per_batch": ms,
            "value": obs.getNrDMs(True) * obs.getNrDMs() * obs.getNrSamplesPerBatch() / ms * 1e3,
            "unit": UNIT}


def bench_subband(torch, device: int, steps: int, hbm_peak: float, peak_adds: float):
    """Config 2 in subband mode (1536 ch in 32 subbands, 64 coarse DMs at 6.4
    x 32 fine DMs at 0.2, 24576 samples, uint8 N(128, 20), 5 % zapped): the
    subband pipeline (packed 16-bit intermediate, dd_subband_run) against the
    engine's two float steps back to back, outputs compared bit for bit."""
    import dedispersion_gb300 as dd
    from dedispersion_gb300 import synthetic as syn
    obs = syn.large_observation(PADDING, subbands=True)
    sh1, sh2 = dd.getShifts(obs, PADDING), dd.getShiftsStepTwo(obs, PADDING)
    zapped = syn.zapped_mask(1536, 0.05, 7, PADDING)
    mapping = syn.identity_mapping(obs, PADDING, subbands=True)
    inp = syn.make_input(obs, 8, PADDING, seed=3, mode=dd.DD_STEP_ONE, mean=128.0, sigma=20.0)
    l1 = dd.layout(obs, dd.DD_STEP_ONE, 8, PADDING)
    l2 = dd.layout(obs, dd.DD_STEP_TWO, 32, PADDING)
    dev = f"cuda:{device}"
    nbuf = 4  # 4 x 45 MB inputs: each step reads its input from HBM
    d_in = [torch.from_numpy(inp).to(dev) for _ in range(nbuf)]
    out = torch.empty(l2.output_bytes // 4, dtype=torch.float32, device=dev)
    ref = torch.empty_like(out)
    pipe = dd.SubbandPipeline(obs, 8, PADDING, device=device)
    pipe.setTables(sh1, sh2, zapped, mapping)
    one = dd.Plan(obs, dd.DD_STEP_ONE, 8, PADDING, device=device)
    one.setShifts(sh1)
    one.setZappedChannels(zapped)
    two = dd.Plan(obs, dd.DD_STEP_TWO, 32, PADDING, device=device)
    two.setShifts(sh2)
    two.setBeamMapping(mapping)
    inter = torch.empty(l1.output_bytes // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def timed(fn):
        for i in range(3):
            fn(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            fn(i)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / steps

    t_pipe = timed(lambda i: pipe.run(d_in[i % nbuf], out, stream))
    pipe.check(stream)
    # consecutive independent batches: step one may start during the previous
    # batch's step two (dd_subband_set_overlap)
    pipe.setOverlap(True)
    t_pipe_ov = timed(lambda i: pipe.run(d_in[i % nbuf], out, stream))
    pipe.check(stream)
    pipe.setOverlap(False)
    # time-chunked runs (dd_subband_set_chunks): the intermediate is read
    # back from L2, at the cost of a partial wave per range
    pipe.setChunks(4)
    t_chunk = timed(lambda i: pipe.run(d_in[i % nbuf], out, stream))
    pipe.check(stream)
    pipe.run(d_in[1], out, stream)
    out_chunked = out.clone()
    pipe.setChunks(0)
    t_float = timed(lambda i: (one.run(d_in[i % nbuf], inter, stream),
                               two.run(inter, ref, stream)))
    two.check(stream)
    pipe.run(d_in[0], out, stream)
    one.run(d_in[0], inter, stream)
    two.run(inter, ref, stream)
    torch.cuda.synchronize()
    exact = bool(torch.equal(out, ref))
    one.run(d_in[1], inter, stream)
    two.run(inter, ref, stream)
    torch.cuda.synchronize()
    exact_chunked = bool(torch.equal(out_chunked, ref))
    info = pipe.info()
    D1, D2, SB = obs.getNrDMs(True), obs.getNrDMs(), obs.getNrSubbands()
    S, S1 = obs.getNrSamplesPerBatch(), obs.getNrSamplesPerBatch(True)
    live = int((zapped[:1536] == 0).sum())
    units = D1 * D2 * S
    adds = live * D1 * S1 + SB * D1 * D2 * S  # step one + step two, algorithmic
    hbm_bytes = inp.nbytes + 2 * info["intermediate_bytes"] + D1 * D2 * S * 4
    for x in (pipe, one, two):
        x.close()
    return {"value": units / t_pipe_ov, "unit": UNIT, "ms_per_batch": t_pipe_ov * 1e3,
            "serial_value": units / t_pipe, "serial_ms_per_batch": t_pipe * 1e3,
            "float_steps_value": units / t_float, "float_steps_ms": t_float * 1e3,
            "speedup_vs_float_steps": t_float / t_pipe, "bit_exact_vs_float_steps": exact,
            "chunked": {"chunks": 4, "ms_per_batch": t_chunk * 1e3, "value": units / t_chunk,
                        "bit_exact_vs_float_steps": exact_chunked,
                        "what": "dd_subband_set_chunks(4): step two in 4 time ranges, each "
                                "right after the step-one tiles it reads, so the intermediate "
                                "is read back from L2 (single-pass ncu: 4.6 MB of DRAM reads "
                                "per batch instead of 87 MB); slower, as both kernels are "
                                "bound by instructions and shared memory"},
            "note_speedup": "serial pipeline against the serial float steps",
            "packed": info["packed"], "intermediate_bytes": info["intermediate_bytes"],
            "adds_per_batch": adds, "adds_frac": adds / t_pipe_ov / peak_adds,
            "hbm_bytes_upper": hbm_bytes,
            "hbm_frac_upper": hbm_bytes / t_pipe_ov / 1e9 / hbm_peak,
            "gpu_launches_per_batch": 2,
            "workload": "1536 ch in 32 subbands (5% zapped), 64 coarse DMs at 6.4 x 32 fine "
                        "DMs at 0.2 = 2048 DMs, 24576 samples, uint8 N(128, 20)",
            "note": "hbm_bytes_upper counts the intermediate written and read once through "
                    "HBM; measured (single-pass ncu), step two reads 87 of its 101 MB from DRAM"}


def _time_batch(torch, device, beams, kernels, reps, persistent=False):
    """One batch over `beams` with per-beam configurations `kernels` (None:
    each beam's default): (ms per batch run, ms per run of the same beams'
    plain launches one after another with the same configurations, whether
    every beam's batch output equals its plain output, batch info)."""
    import dedispersion_gb300 as dd
    batch = dd.Batch(device)
    plans = []
    for (sh, obs, shifts, zapped, mapping, d_in, lay, d_out, d_ref), k in zip(beams, kernels):
        batch.add(obs, sh["bits"], PADDING, shifts, zapped, mapping, d_in, d_out, kernel=k)
        plan = dd.Plan(obs, dd.DD_SINGLE_STEP, sh["bits"], PADDING, device=device, kernel=k)
        plan.setShifts(shifts)
        plan.setZappedChannels(zapped)
        plan.setBeamMapping(mapping)
        plans.append(plan)
    if persistent:
        batch.setPersistent(True)
    batch.commit()
    stream = torch.cuda.current_stream()
    batch.run(stream)
    batch.check(stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        batch.run(stream)
    e1.record(stream)
    batch.check(stream)
    t_batch = e0.elapsed_time(e1) / reps
    for b, plan in zip(beams, plans):
        plan.run(b[5], b[8], stream)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        for b, plan in zip(beams, plans):
            plan.run(b[5], b[8], stream)
    e1.record(stream)
    torch.cuda.synchronize()
    t_plain = e0.elapsed_time(e1) / reps
    exact = True
    for (sh, obs, shifts, zapped, mapping, d_in, lay, d_out, d_ref), plan in zip(beams, plans):
        S = obs.getNrSamplesPerBatch()
        rows = lay.output_bytes // 4 // lay.output_row_elems
        exact &= bool(torch.equal(d_out.view(rows, -1)[:, :S], d_ref.view(rows, -1)[:, :S]))
        plan.close()
    info = batch.info()
    batch.close()
    return t_batch, t_plain, exact, info


def bench_batched(torch, device: int, reps: int = 3, count: int = 40, peak_adds: float = 0.0):
    """40 uneven beams (384/1536 ch, 8192-32768 samples, 512-4096 DMs, steps
    0.1-0.5, 2/4/8-bit uniform input) in one CUDA graph launch (the beams'
    kernels forked over concurrent branches), against the same beams launched
    one plain kernel each on one stream.  Each beam's configuration is picked
    by timing a shortlist on it before the batch is recorded
    (tuning.batch_candidates; outside the timed region); the same batch with
    each beam's default configuration is reported beside it."""
    import dedispersion_gb300 as dd
    from dedispersion_gb300 import synthetic as syn
    from dedispersion_gb300 import tuning
    shapes = syn.batched_shapes(count)
    beams = []
    units = adds = 0
    for sh in shapes:
        obs = syn.shape_observation(sh, PADDING)
        shifts = dd.getShifts(obs, PADDING)
        zapped = syn.zapped_mask(sh["channels"], 0.05, sh["seed"], PADDING)
        mapping = syn.identity_mapping(obs, PADDING)
        d_in = syn.device_uniform_input(torch, obs, sh["bits"], PADDING, sh["seed"])
        lay = dd.layout(obs, dd.DD_SINGLE_STEP, sh["bits"], PADDING)
        d_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32, device=f"cuda:{device}")
        d_ref = torch.empty_like(d_out)
        beams.append((sh, obs, shifts, zapped, mapping, d_in, lay, d_out, d_ref))
        units += obs.getNrDMs() * obs.getNrSamplesPerBatch()
        adds += obs.getNrDMs() * obs.getNrSamplesPerBatch() * int((zapped[:sh["channels"]] == 0).sum())
    t0 = time.perf_counter()
    picks = [tuning.pick(b[1], b[0]["bits"], PADDING, b[2], b[3], b[4], b[5], b[7], device=device)
             for b in beams]
    t_tune = time.perf_counter() - t0
    kernels = [p.kernel for p in picks]
    t_batch, t_plain, exact, info = _time_batch(torch, device, beams, kernels, reps)
    d_batch, d_plain, d_exact, _ = _time_batch(torch, device, beams, [None] * len(beams), reps)
    p_batch, _, p_exact, p_info = _time_batch(torch, device, beams, [None] * len(beams), reps,
                                              persistent=True)
    shared = info.get("form") == "graph"
    return {"value": units / t_batch * 1e3, "unit": UNIT, "ms_per_batch": t_batch,
            "plain_sequential_value": units / t_plain * 1e3, "plain_sequential_ms": t_plain,
            "speedup_vs_plain": t_plain / t_batch, "beams": count, "tiles": info["tiles"],
            "adds_per_batch": adds,
            "adds_frac": adds / t_batch * 1e3 / peak_adds if peak_adds else None,
            ("branches" if shared else "persistent_ctas"): info["grid"],
            "form": info.get("form"), "bit_exact_vs_plain": exact and d_exact and p_exact,
            "tiles_picked_by": f"timing {len(tuning.batch_candidates())} shortlisted "
                               f"configurations per beam before recording ({t_tune:.1f} s)",
            "picked": {name: sum(p.name == name for p in picks)
                       for name in sorted({p.name for p in picks})},
            "default_tiles": {"ms_per_batch": d_batch, "value": units / d_batch * 1e3,
                              "plain_sequential_ms": d_plain,
                              "adds_frac": adds / d_batch * 1e3 / peak_adds if peak_adds else None},
            "persistent_form": {"ms_per_batch": p_batch, "value": units / p_batch * 1e3,
                                "adds_frac": adds / p_batch * 1e3 / peak_adds if peak_adds else None,
                                "ctas": p_info["grid"],
                                "what": "one persistent direct-tile kernel over all 40 beams' "
                                        "tiles, replayed from a CUDA graph"},
            "launch": ("one CUDA graph: the beams' kernels on concurrent branches" if shared
                       else "one persistent kernel replayed from a CUDA graph"),
            "workload": "40 beams: 384/1536 ch, 8192-32768 samples, 512-4096 DMs, DM step "
                        "0.1-0.5, 2/4/8-bit uniform input, 5% zapped"}


def served_adds(server):
    """Algorithmic adds of one batch of every admitted beam: live channels x
    DMs x samples for a single-step beam; step one (live channels x coarse
    DMs x step-one samples) plus step two (subbands x DMs x samples) for a
    subband beam."""
    import dedispersion_gb300 as dd
    total = 0
    for st in server.streams:
        cfg = st.cfg
        live = int((st.zapped[:cfg.channels] == 0).sum())
        if cfg.subband:
            d1 = cfg.dms // cfg.dms_per_subband_dm
            tail2 = dd.layout(st.obs, dd.DD_STEP_TWO, 32, cfg.padding, st.shifts2).max_delay
            total += live * d1 * (cfg.samples + tail2) + cfg.subbands * cfg.dms * cfg.samples
        else:
            total += live * cfg.dms * cfg.samples
    return total


def bench_served(device: int, batches: int = 12, compression: float = 16.0,
                 double_buffer: bool = True, runs: int = 3, peak_adds: float = 0.0):
    """12 beams streaming 2.048 s batches (1536 ch, 25000 samples at 81.92 us,
    8-bit), DM ranges of 1024-4096 DMs at step 0.2, alternating single-step and
    subband (32 subbands) modes, admitted against a 150 GB budget.  After a
    warm-up that pushes every staging buffer of every beam once, `runs` runs
    of each: Poisson-jittered arrivals on a clock 16x faster than real time
    (latency), and all batches at once (throughput); medians and spreads."""
    from dedispersion_gb300 import serving
    cfgs = serving.served_beams(12, seed=77, padding=PADDING, double_buffer=double_buffer)
    server = serving.Server(budget_bytes=150 * 10**9, device=device)
    for c in cfgs:
        server.admit(c)
    data = []
    for c in cfgs:
        g = np.random.default_rng(c.seed)
        data.append([g.integers(0, 256, size=(c.channels, c.samples), dtype=np.uint8)
                     for _ in range(2)])

    def source(b, k, staging):
        np.copyto(staging[:, :cfgs[b].samples], data[b][k % 2])

    period = cfgs[0].period
    nbuf = max(s.nbuf for s in server.streams)
    # warm-up: every staging buffer (and so every recorded graph) of every beam
    server.serve([(0.0, b, k) for k in range(nbuf) for b in range(len(cfgs))], source)
    lat_runs, thr_runs = [], []
    for r in range(runs):
        sched = serving.poisson_schedule(len(cfgs), batches, period, 0.1 * period, seed=9 + r)
        lat_runs.append(server.serve(sched, source, time_compression=compression,
                                     deadline=period).summary())
        thr_runs.append(server.serve([(0.0, b, k) for k in range(batches)
                                      for b in range(len(cfgs))], source,
                                     deadline=period).summary())
    med = lambda xs: float(statistics.median(xs))  # noqa: E731
    thr = [t["throughput_dm_samples_per_s"] for t in thr_runs]
    p50 = [t["p50_latency_s"] for t in lat_runs]
    p99 = [t["p99_latency_s"] for t in lat_runs]
    units_per_round = sum(st.dm_samples for st in server.streams)
    adds_per_round = served_adds(server)
    value = med(thr)
    out = {"value": value, "unit": UNIT, "runs": runs,
           "value_spread": [min(thr), max(thr)],
           "p50_latency_s": med(p50), "p50_spread_s": [min(p50), max(p50)],
           "p99_latency_s": med(p99), "p99_spread_s": [min(p99), max(p99)],
           "max_latency_s": max(t["max_latency_s"] for t in lat_runs), "deadline_s": period,
           "deadline_misses": sum(t["deadline_misses"] for t in lat_runs),
           "batches_per_run": lat_runs[0]["batches"],
           "time_compression": compression,
           "offered_load_throughput": med([t["throughput_dm_samples_per_s"] for t in lat_runs]),
           "beams": len(cfgs), "subband_beams": sum(c.subband for c in cfgs),
           "adds_per_round": adds_per_round,
           "adds_frac": (value / units_per_round * adds_per_round / peak_adds
                         if peak_adds else None),
           "admitted_device_bytes": server.used, "budget_bytes": server.budget,
           "double_buffered": double_buffer,
           "workload": "12 beams x 25000-sample 8-bit batches, 1536 ch, 1024-4096 DMs at 0.2, "
                       "single-step and 32-subband streams, tail carried on the device; value = "
                       "median over runs of all batches queued at once, latency = "
                       "Poisson-jittered arrivals at 16x real time, host-in to host-out"}
    server.close()
    return out


def run_reference(args, rank, world):
    """The CPU arm: the oracle port (a loop-for-loop port of the reference's
    dedispersion, bit-identical to it) on every host thread, each step a DM
    prefix of the workload.  Built from numpy and the oracle alone: the
    engine's library is never loaded in this process."""
    if rank != 0:
        return
    from oracle import workload as owl
    o, sh, z, m, inp = owl.single_step(seed=beam_seed(0), padding=PADDING)
    threads = os.cpu_count() or 1
    import oracle
    out = np.zeros(o.nr_dms * out_row(o), dtype=np.float32)
    # size one step's DM prefix for ~1/(steps+warmup) of a ~60 s budget
    _, dms, dt = cpu_sample(o, sh, z, m, inp, max(0.5, 60.0 / (args.steps + args.warmup)),
                            threads)
    for _ in range(args.warmup):
        oracle.dedispersion(o, z, m, inp, out, sh, PADDING, 8, 0, dms, threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        oracle.dedispersion(o, z, m, inp, out, sh, PADDING, 8, 0, dms, threads)
    elapsed = time.perf_counter() - t
    value = args.steps * dms * o.nr_samples_per_batch / elapsed
    sample = (f"DMs 0..{dms - 1} of 2048 x 24576 samples x 1536 channels per step "
              f"(same delays as the full workload)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic", "config": {"workload": WORKLOAD, "dm_prefix": dms},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own CPU code needs its sources, which are not on the GPU "
                "machine; the port timed here equals it bit for bit (tests/test_oracle.py)",
    }), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1 and args.impl == "reference" and rank != 0:
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import dedispersion_gb300 as dd
    torch.cuda.set_device(local)
    if args.served_only:
        rates = dd.measure_add_rate(local, 2)
        print(json.dumps(bench_served(local, peak_adds=max(rates.values()))))
        return
    if args.float_only:
        rates = dd.measure_add_rate(local, 2)
        print(json.dumps(bench_float(torch, local, args.steps,
                                     max(rates["fadd_per_s"], rates["iadd_per_s"]),
                                     args.float_kernel, args.float_dms)))
        return
    if args.subband_only is not None:
        print(json.dumps(subband_only(torch, local, args.subband_only, args.steps, args.warmup)))
        return
    pg = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = tdist

    obs, shifts, zapped, mapping, inp = workload(seed=beam_seed(rank))
    S, D = obs.getNrSamplesPerBatch(), obs.getNrDMs()
    live = int((zapped[:1536] == 0).sum())
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, PADDING, shifts)
    kidx = None
    if args.kernel:
        kidx = next((k.index for k in dd.kernels() if k.name == args.kernel), None)
        if kidx is None:
            raise SystemExit(f"no compiled configuration named {args.kernel}")
    plan = dd.Plan(obs, dd.DD_SINGLE_STEP, 8, PADDING, device=local, kernel=kidx)
    plan.setShifts(shifts)
    plan.setZappedChannels(zapped)
    plan.setBeamMapping(mapping)
    # Consecutive steps are independent batches: each launch may start on the
    # SMs the previous launch's last wave leaves idle (dd_plan_set_overlap).
    plan.setOverlap(True)
    nbuf = 4
    d_in = [torch.from_numpy(inp).to(f"cuda:{local}") for _ in range(nbuf)]
    d_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    for i in range(args.warmup):
        plan.run(d_in[i % nbuf], d_out, stream)
    plan.check(stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for i in range(args.steps):
            plan.run(d_in[i % nbuf], d_out, stream)
        e1.record(stream)
        barrier()
        # keep the GPU busy for the clock sampler if the timed region was short
        ms = e0.elapsed_time(e1)
    plan.check(stream)
    clocks = clk.summary()
    t_dev = max_over_ranks(ms / 1e3, pg, f"cuda:{local}")
    value = job_value(world, args.steps, D, S, t_dev)
    per_launch_s = t_dev / args.steps
    # The same steps launched one after another (no overlap), for comparison.
    plan.setOverlap(False)
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e2.record(stream)
    for i in range(args.steps):
        plan.run(d_in[i % nbuf], d_out, stream)
    e3.record(stream)
    barrier()
    plan.check(stream)
    plan.setOverlap(True)
    t_serial = max_over_ranks(e2.elapsed_time(e3) / 1e3, pg, f"cuda:{local}")
    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": t_dev / args.steps * 1e3, "kernel_only": True,
                              "kernel_conf": plan.conf().print(),
                              "gpu_launches": args.steps * plan.launches()}), flush=True)
        return

    sm_mhz = clocks.get("sm_mhz") or 2070.0
    formula_adds = SMS * LANES * sm_mhz * 1e6
    # The add roofline's denominator, measured on this GPU now: the faster of
    # a float-add and an integer-add stream over every SM (dd_measure_add_rate).
    with ClockSampler(local) as peak_clk:
        rates = dd.measure_add_rate(local, 3)
    peak_clocks = peak_clk.summary()
    peak_adds = max(rates["fadd_per_s"], rates["iadd_per_s"])
    hbm_peak = 6784.2
    try:
        hbm_peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"]
    except Exception:
        pass
    # The served line runs first among the extra lines: its latencies are
    # host-driven, and later lines leave large pinned host arrays and many
    # plans behind.
    gc.collect()
    served = bench_served(local, peak_adds=peak_adds) if not args.no_served else None
    # e2e through the C ABI's synchronous host-buffer call, pinned host memory
    h_in = torch.from_numpy(inp).pin_memory()
    h_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32).pin_memory()
    in_np, out_np = h_in.numpy(), h_out.numpy()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        dd.dedispersion(obs, zapped, mapping, in_np, out_np, shifts, PADDING, 8)
    barrier()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        dd.dedispersion(obs, zapped, mapping, in_np, out_np, shifts, PADDING, 8)
    barrier()
    t_e2e = max_over_ranks(time.perf_counter() - t, pg, f"cuda:{local}")
    e2e_value = job_value(world, e2e_steps, D, S, t_e2e)

    detect = bench_detect(torch, plan, d_in, d_out, stream, D, S, args.steps)
    ingest_line = bench_ingest(torch, inp, lay, obs, stream)
    subband = bench_subband(torch, local, max(10, min(args.steps, 50)), hbm_peak, peak_adds)
    float32 = bench_float(torch, local, max(3, min(args.steps, 10)), peak_adds, args.float_kernel)
    batched = bench_batched(torch, local, peak_adds=peak_adds) if not args.no_batched else None
    tuning_line = None
    if not args.no_tuning:
        from dedispersion_gb300 import tuning
        tuning_line = tuning.bench_report(device=local)

    if rank != 0:
        return
    # roofline of the plain kernel
    adds_per_launch = D * S * live
    achieved_adds = adds_per_launch / per_launch_s
    compulsory = inp.nbytes // 1 + D * S * 4
    traffic = read_profile_traffic()
    executed_adds = plan.adds()
    kernel_name = next((k.name for k in dd.kernels()
                        if k.conf.print() == plan.conf().print()), plan.conf().print())
    cpu_line = cpu_baseline(obs.c, shifts, zapped, mapping, inp, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "padding": PADDING, "live_channels": live,
                   "kernel_conf": plan.conf().print(),
                   "l2": "inputs rotate over 4 device buffers (4 x 45 MB) and each step writes "
                         "201 MB of output, so every step reads its input from HBM",
                   "parallelism": f"{world} independent beams (one per GPU)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(inp.nbytes),
                "d2h_bytes_per_step": int(D * S * 4),
                "call": "dd_dedispersion (C ABI, synchronous, host buffers)"},
        "roofline": {"bound": "alu", "achieved": achieved_adds / 1e9, "peak": peak_adds / 1e9,
                     "unit": "Gadd/s", "frac": achieved_adds / peak_adds,
                     "traffic": traffic,
                     "peak_source": "measured: the faster of a float-add and a 32-bit "
                                    "integer-add stream over every SM, timed with CUDA events "
                                    "in this run (dd_measure_add_rate)",
                     "peak_measured": {"fadd_per_s": rates["fadd_per_s"],
                                       "iadd_per_s": rates["iadd_per_s"],
                                       "sm_mhz": peak_clocks.get("sm_mhz"),
                                       "reasons": peak_clocks.get("reasons")},
                     "peak_formula": {"adds_per_s": formula_adds,
                                      "what": f"{SMS} SMs x {LANES} lanes x {sm_mhz:.0f} MHz "
                                              "(median SM clock of the timed region)"},
                     "adds_per_launch": adds_per_launch,
                     "kernel": kernel_name,
                     "executed": {
                         "adds_per_launch": executed_adds,
                         "achieved": executed_adds / per_launch_s / 1e9,
                         "frac": executed_adds / per_launch_s / peak_adds,
                         "note": "integer adds the kernel performs (partial sums shared by "
                                 "DMs with equal relative delays + series adds); the "
                                 "direct-sum count above is the algorithmic work"},
                     "hbm": {"achieved_gbs": compulsory / per_launch_s / 1e9,
                             "peak_gbs": hbm_peak,
                             "frac": compulsory / per_launch_s / 1e9 / hbm_peak,
                             "compulsory_bytes_per_launch": compulsory}},
        "cpu_baseline": cpu_line,
        "clocks": clocks,
        "gpu_launches": args.steps * plan.launches(),
        "serial_launches": {"ms_per_step": t_serial / args.steps * 1e3,
                            "value": job_value(world, args.steps, D, S, t_serial),
                            "what": "the same steps with dd_plan_set_overlap off: each launch "
                                    "starts after the previous one completes"},
        "detect": detect,
        "ingest": ingest_line,
        "subband": subband,
        "float32": float32,
        "batched": batched,
        "served": served,
        "tuning": tuning_line,
    }
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
