"""GB300-native incoherent dedispersion.

Host-side mirror of TRASAL/Dedispersion's interface for the dedispersion
path, over the C ABI of ``libdedisp_gb300.so`` (include/dedisp_gb300.h):

* :class:`Observation` -- the AstroData::Observation setters and getters the
  reference uses (include/Dedispersion.hpp, src/Shifts.cpp).
* :class:`DedispersionConf` -- Dedispersion::DedispersionConf
  (include/Dedispersion.hpp:34-54).
* :func:`getShifts`, :func:`getShiftsStepTwo` -- src/Shifts.cpp:20-42.
* :func:`dedispersion`, :func:`subbandDedispersionStepOne`,
  :func:`subbandDedispersionStepTwo` -- include/Dedispersion.hpp:59-61: same
  argument order and meaning; ``output`` is filled in place.  They run on the
  GPU (sm_103a kernels); without a GPU they raise ``DedispersionError`` with
  status ``DD_ERR_NO_DEVICE``.  There is no CPU fallback.
* :func:`readTunedDedispersionConf` -- src/Dedispersion.cpp:20-81.
* :class:`Plan` -- device-resident tables and asynchronous launches on device
  pointers (the twin of the generated OpenCL kernels).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import (DD_SINGLE_STEP, DD_STEP_ONE, DD_STEP_TWO, DdConf, DdLayout,
                   DdObservation, DedispersionError, check, lib)

__all__ = [
    "Observation", "DedispersionConf", "DedispersionError", "Plan", "getShifts",
    "getShiftsStepTwo", "dedispersion", "subbandDedispersionStepOne",
    "subbandDedispersionStepTwo", "readTunedDedispersionConf", "writeTunedDedispersionConf",
    "layout", "pad", "DD_SINGLE_STEP", "DD_STEP_ONE", "DD_STEP_TWO", "device_count",
]


def pad(value: int, padding: int) -> int:
    """isa::utils::pad: round up to a multiple of ``padding`` (0 = unchanged)."""
    return int(lib().dd_pad(int(value), int(padding)))


def measure_add_rate(device: int = 0, repeats: int = 3) -> dict:
    """Measured float and 32-bit integer add throughput of a GPU, adds/s
    (dd_measure_add_rate): the denominator of the add roofline."""
    f, i = C.c_double(0), C.c_double(0)
    check(lib().dd_measure_add_rate(device, repeats, C.byref(f), C.byref(i)))
    return {"fadd_per_s": f.value, "iadd_per_s": i.value}


def device_count() -> int:
    n = C.c_int(0)
    check(lib().dd_device_count(C.byref(n)))
    return n.value


class Observation:
    """AstroData::Observation, restricted to the state the dedispersion path
    reads.  Setter/getter names and argument order follow AstroData."""

    def __init__(self) -> None:
        self._c = DdObservation()
        self._c.nr_beams = 1
        self._c.nr_synthesized_beams = 1
        self._c.nr_subbands = 1
        self._c.downsampling = 1

    # -- setters
    def setNrBeams(self, n: int) -> None:
        self._c.nr_beams = n

    def setNrSynthesizedBeams(self, n: int) -> None:
        self._c.nr_synthesized_beams = n

    def setNrSamplesPerBatch(self, n: int, subbanding: bool = False) -> None:
        if subbanding:
            self._c.nr_samples_per_batch_subbanding = n
        else:
            self._c.nr_samples_per_batch = n

    def setNrSamplesPerDispersedBatch(self, n: int, subbanding: bool = False) -> None:
        if subbanding:
            self._c.nr_samples_per_dispersed_batch_subbanding = n
        else:
            self._c.nr_samples_per_dispersed_batch = n

    def setSamplingTime(self, t: float) -> None:
        self._c.sampling_time = t

    def setFrequencyRange(self, nrSubbands: int, nrChannels: int, minFreq: float,
                          channelBandwidth: float) -> None:
        self._c.nr_subbands = nrSubbands
        self._c.nr_channels = nrChannels
        self._c.min_freq = minFreq
        self._c.channel_bandwidth = channelBandwidth

    def setDMRange(self, nrDMs: int, firstDM: float, step: float,
                   subbanding: bool = False) -> None:
        if subbanding:
            self._c.nr_dms_subbanding = nrDMs
            self._c.first_dm_subbanding = firstDM
            self._c.dm_step_subbanding = step
        else:
            self._c.nr_dms = nrDMs
            self._c.first_dm = firstDM
            self._c.dm_step = step

    def setNrZappedChannels(self, n: int) -> None:
        self._c.nr_zapped_channels = n

    # -- getters
    def getNrBeams(self) -> int:
        return self._c.nr_beams

    def getNrSynthesizedBeams(self) -> int:
        return self._c.nr_synthesized_beams

    def getNrSamplesPerBatch(self, subbanding: bool = False, padding: int = 0) -> int:
        v = self._c.nr_samples_per_batch_subbanding if subbanding else self._c.nr_samples_per_batch
        return pad(v, padding)

    def getNrSamplesPerDispersedBatch(self, subbanding: bool = False, padding: int = 0) -> int:
        v = (self._c.nr_samples_per_dispersed_batch_subbanding if subbanding
             else self._c.nr_samples_per_dispersed_batch)
        return pad(v, padding)

    def getNrChannels(self, padding: int = 0) -> int:
        return pad(self._c.nr_channels, padding)

    def getNrSubbands(self, padding: int = 0) -> int:
        return pad(self._c.nr_subbands, padding)

    def getNrChannelsPerSubband(self) -> int:
        return self._c.nr_channels // self._c.nr_subbands

    def getNrZappedChannels(self) -> int:
        return self._c.nr_zapped_channels

    def getNrDMs(self, subbanding: bool = False) -> int:
        return self._c.nr_dms_subbanding if subbanding else self._c.nr_dms

    def getFirstDM(self, subbanding: bool = False) -> float:
        return self._c.first_dm_subbanding if subbanding else self._c.first_dm

    def getDMStep(self, subbanding: bool = False) -> float:
        return self._c.dm_step_subbanding if subbanding else self._c.dm_step

    def getSamplingTime(self) -> float:
        return self._c.sampling_time

    def getDownsampling(self) -> int:
        return self._c.downsampling

    def getMinFreq(self) -> float:
        return self._c.min_freq

    def getChannelBandwidth(self) -> float:
        return self._c.channel_bandwidth

    def getMaxFreq(self) -> float:
        return lib().dd_max_freq(C.byref(self._c))

    def getSubbandMinFreq(self) -> float:
        return lib().dd_subband_min_freq(C.byref(self._c))

    def getSubbandMaxFreq(self) -> float:
        return lib().dd_subband_max_freq(C.byref(self._c))

    def getSubbandBandwidth(self) -> float:
        return lib().dd_subband_bandwidth(C.byref(self._c))

    @property
    def c(self) -> DdObservation:
        """The C struct the ABI takes."""
        return self._c

    def copy(self) -> "Observation":
        o = Observation()
        C.memmove(C.byref(o._c), C.byref(self._c), C.sizeof(DdObservation))
        return o


@dataclass
class DedispersionConf:
    """Dedispersion::DedispersionConf and the KernelConf fields it extends."""

    splitBatches: bool = False
    localMem: bool = True
    unroll: int = 8
    nrThreadsD0: int = 32
    nrThreadsD1: int = 8
    nrThreadsD2: int = 1
    nrItemsD0: int = 16
    nrItemsD1: int = 4
    nrItemsD2: int = 1

    def getSplitBatches(self) -> bool: return self.splitBatches
    def getLocalMem(self) -> bool: return self.localMem
    def getUnroll(self) -> int: return self.unroll
    def setSplitBatches(self, v: bool) -> None: self.splitBatches = bool(v)
    def setLocalMem(self, v: bool) -> None: self.localMem = bool(v)
    def setUnroll(self, v: int) -> None: self.unroll = int(v)
    def getNrThreadsD0(self) -> int: return self.nrThreadsD0
    def getNrThreadsD1(self) -> int: return self.nrThreadsD1
    def getNrThreadsD2(self) -> int: return self.nrThreadsD2
    def getNrItemsD0(self) -> int: return self.nrItemsD0
    def getNrItemsD1(self) -> int: return self.nrItemsD1
    def getNrItemsD2(self) -> int: return self.nrItemsD2
    def setNrThreadsD0(self, v: int) -> None: self.nrThreadsD0 = int(v)
    def setNrThreadsD1(self, v: int) -> None: self.nrThreadsD1 = int(v)
    def setNrThreadsD2(self, v: int) -> None: self.nrThreadsD2 = int(v)
    def setNrItemsD0(self, v: int) -> None: self.nrItemsD0 = int(v)
    def setNrItemsD1(self, v: int) -> None: self.nrItemsD1 = int(v)
    def setNrItemsD2(self, v: int) -> None: self.nrItemsD2 = int(v)

    def to_c(self) -> DdConf:
        return DdConf(int(self.splitBatches), int(self.localMem), self.unroll, self.nrThreadsD0,
                      self.nrThreadsD1, self.nrThreadsD2, self.nrItemsD0, self.nrItemsD1,
                      self.nrItemsD2)

    @classmethod
    def from_c(cls, c: DdConf) -> "DedispersionConf":
        return cls(bool(c.split_batches), bool(c.local_mem), c.unroll, c.threads_d0, c.threads_d1,
                   c.threads_d2, c.items_d0, c.items_d1, c.items_d2)

    def print(self) -> str:
        """'split local unroll tD0 tD1 tD2 iD0 iD1 iD2' (src/Dedispersion.cpp:87-89)."""
        buf = C.create_string_buffer(256)
        c = self.to_c()
        check(lib().dd_conf_print(C.byref(c), buf, 256))
        return buf.value.decode()

    @classmethod
    def default(cls, observation: Observation, mode: int, inputBits: int) -> "DedispersionConf":
        c = DdConf()
        check(lib().dd_default_conf(C.byref(observation.c), mode, inputBits, C.byref(c)))
        return cls.from_c(c)


def _shift_table(fn, observation: Observation, padding: int, n: int) -> np.ndarray:
    cap = pad(n, padding // 4) + 1
    out = np.zeros(cap, dtype=np.float32)
    check(fn(C.byref(observation.c), padding, out.ctypes.data_as(C.POINTER(C.c_float)), cap))
    return out[:cap - 1].copy()


def getShifts(observation: Observation, padding: int) -> np.ndarray:
    """Per-channel delay in samples per unit DM (src/Shifts.cpp:20-30)."""
    return _shift_table(lib().dd_get_shifts, observation, padding, observation.getNrChannels())


def getShiftsStepTwo(observation: Observation, padding: int) -> np.ndarray:
    """Per-subband delay in samples per unit DM (src/Shifts.cpp:32-42)."""
    return _shift_table(lib().dd_get_shifts_step_two, observation, padding,
                        observation.getNrSubbands())


def layout(observation: Observation, mode: int, inputBits: int, padding: int,
           shifts: np.ndarray | None = None) -> DdLayout:
    """Row pitches and buffer sizes of one mode in the reference layout."""
    out = DdLayout()
    sp = None
    if shifts is not None:
        sh = np.ascontiguousarray(shifts, dtype=np.float32)
        sp = sh.ctypes.data_as(C.POINTER(C.c_float))
    check(lib().dd_get_layout(C.byref(observation.c), mode, inputBits, padding, sp, C.byref(out)))
    return out


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _ptr(a: np.ndarray, ct=C.c_void_p):
    return a.ctypes.data_as(C.POINTER(ct)) if ct is not C.c_void_p else C.c_void_p(a.ctypes.data)


def _check_buffers(inp: np.ndarray, out: np.ndarray, lay: DdLayout) -> None:
    if inp.nbytes < lay.input_bytes:
        raise DedispersionError(_abi.DD_ERR_INVALID_ARGUMENT,
                                f"input holds {inp.nbytes} bytes, layout needs {lay.input_bytes}")
    if out.dtype != np.float32 or not out.flags.c_contiguous or not out.flags.writeable:
        raise DedispersionError(_abi.DD_ERR_INVALID_ARGUMENT,
                                "output must be a writable C-contiguous float32 array")
    if out.nbytes < lay.output_bytes:
        raise DedispersionError(_abi.DD_ERR_INVALID_ARGUMENT,
                                f"output holds {out.nbytes} bytes, layout needs {lay.output_bytes}")


def dedispersion(observation: Observation, zappedChannels, beamMapping, input: np.ndarray,
                 output: np.ndarray, shifts, padding: int, inputBits: int) -> None:
    """Dedispersion::dedispersion (include/Dedispersion.hpp:59, 70-109)."""
    inp = np.ascontiguousarray(input)
    lay = layout(observation, DD_SINGLE_STEP, inputBits, padding)
    _check_buffers(inp, output, lay)
    z, m = _u32(zappedChannels), _u32(beamMapping)
    sh = np.ascontiguousarray(shifts, dtype=np.float32)
    check(lib().dd_dedispersion(C.byref(observation.c), _ptr(z, C.c_uint32), _ptr(m, C.c_uint32),
                                _ptr(inp), _ptr(output, C.c_float), _ptr(sh, C.c_float), padding,
                                inputBits))


def subbandDedispersionStepOne(observation: Observation, zappedChannels, input: np.ndarray,
                               output: np.ndarray, shifts, padding: int, inputBits: int) -> None:
    """Dedispersion::subbandDedispersionStepOne (include/Dedispersion.hpp:60, 111-153)."""
    inp = np.ascontiguousarray(input)
    lay = layout(observation, DD_STEP_ONE, inputBits, padding)
    _check_buffers(inp, output, lay)
    z = _u32(zappedChannels)
    sh = np.ascontiguousarray(shifts, dtype=np.float32)
    check(lib().dd_subband_dedispersion_step_one(C.byref(observation.c), _ptr(z, C.c_uint32),
                                                 _ptr(inp), _ptr(output, C.c_float),
                                                 _ptr(sh, C.c_float), padding, inputBits))


def subbandDedispersionStepTwo(observation: Observation, beamMapping, input: np.ndarray,
                               output: np.ndarray, shifts, padding: int) -> None:
    """Dedispersion::subbandDedispersionStepTwo (include/Dedispersion.hpp:61, 155-176)."""
    inp = np.ascontiguousarray(input, dtype=np.float32)
    lay = layout(observation, DD_STEP_TWO, 32, padding)
    _check_buffers(inp, output, lay)
    m = _u32(beamMapping)
    sh = np.ascontiguousarray(shifts, dtype=np.float32)
    check(lib().dd_subband_dedispersion_step_two(C.byref(observation.c), _ptr(m, C.c_uint32),
                                                 _ptr(inp, C.c_float), _ptr(output, C.c_float),
                                                 _ptr(sh, C.c_float), padding))


def subbandDedispersion(observation: Observation, zappedChannels, beamMapping, input: np.ndarray,
                        output: np.ndarray, shifts, shiftsStepTwo, padding: int,
                        inputBits: int) -> None:
    """subbandDedispersionStepOne followed by subbandDedispersionStepTwo
    (include/Dedispersion.hpp:60-61) in one call, the intermediate kept on the
    device (packed 16-bit sums where they fit); input in step one's layout,
    output in step two's, equal to the two calls bit for bit."""
    inp = np.ascontiguousarray(input)
    l1 = layout(observation, DD_STEP_ONE, inputBits, padding)
    l2 = layout(observation, DD_STEP_TWO, 32, padding)
    _check_buffers(inp, output, DdLayout(input_row_bytes=l1.input_row_bytes,
                                         input_bytes=l1.input_bytes,
                                         output_row_elems=l2.output_row_elems,
                                         output_bytes=l2.output_bytes))
    z, m = _u32(zappedChannels), _u32(beamMapping)
    sh = np.ascontiguousarray(shifts, dtype=np.float32)
    sh2 = np.ascontiguousarray(shiftsStepTwo, dtype=np.float32)
    check(lib().dd_subband_dedispersion(C.byref(observation.c), _ptr(z, C.c_uint32),
                                        _ptr(m, C.c_uint32), _ptr(inp), _ptr(output, C.c_float),
                                        _ptr(sh, C.c_float), _ptr(sh2, C.c_float), padding,
                                        inputBits))


class SubbandPipeline:
    """Device pipeline of the subband method (dd_subband_*): step one then
    step two on device buffers, the intermediate owned by the pipeline."""

    def __init__(self, observation: Observation, inputBits: int, padding: int, device: int = 0):
        self.observation = observation.copy()
        self.inputBits, self.padding = inputBits, padding
        self._h = C.c_void_p()
        check(lib().dd_subband_create(C.byref(self._h), C.byref(self.observation.c), inputBits,
                                      padding, device))
        self.layout_in = layout(self.observation, DD_STEP_ONE, inputBits, padding)
        self.layout_out = layout(self.observation, DD_STEP_TWO, 32, padding)

    def setTables(self, shifts, shiftsStepTwo, zapped, mapping) -> None:
        sh = np.ascontiguousarray(shifts, dtype=np.float32)
        sh2 = np.ascontiguousarray(shiftsStepTwo, dtype=np.float32)
        z, m = _u32(zapped), _u32(mapping)
        check(lib().dd_subband_set_tables(self._h, _ptr(sh, C.c_float), sh.size,
                                          _ptr(sh2, C.c_float), sh2.size,
                                          _ptr(z, C.c_uint32), z.size, _ptr(m, C.c_uint32),
                                          m.size))

    def setOverlap(self, enable: bool = True) -> None:
        """Let step one of each run start while the previous run's step two
        finishes (dd_subband_set_overlap): consecutive independent runs only."""
        check(lib().dd_subband_set_overlap(self._h, 1 if enable else 0))

    def setChunks(self, chunks: int) -> None:
        """Run the two steps interleaved over `chunks` time ranges so that the
        intermediate is read back from L2 (dd_subband_set_chunks); 0 or 1:
        each step in one launch."""
        check(lib().dd_subband_set_chunks(self._h, int(chunks)))

    def setPairKernel(self, index: int) -> None:
        check(lib().dd_subband_set_pair_kernel(self._h, int(index)))

    def run(self, d_input, d_output, stream=None) -> None:
        check(lib().dd_subband_run(self._h, C.c_void_p(_devptr(d_input)),
                                   C.c_void_p(_devptr(d_output)), C.c_void_p(_stream(stream))))

    def check(self, stream=None) -> None:
        check(lib().dd_subband_check(self._h, C.c_void_p(_stream(stream))))

    def info(self) -> dict:
        packed, nbytes = C.c_int(0), C.c_uint64(0)
        check(lib().dd_subband_info(self._h, C.byref(packed), C.byref(nbytes)))
        return {"packed": bool(packed.value), "intermediate_bytes": nbytes.value}

    def close(self) -> None:
        if self._h:
            lib().dd_subband_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self) -> "SubbandPipeline":
        return self

    def __exit__(self, *exc) -> None:
        self.close()


def pair_kernel_count() -> int:
    return int(lib().dd_subband_pair_kernel_count())


def readTunedDedispersionConf(filename: str, device: str, nrDMs: int) -> DedispersionConf:
    """The (device, nrDMs) entry of a tuned-configuration file
    (src/Dedispersion.cpp:20-81).  Raises DedispersionError(DD_ERR_FILE) if the
    file cannot be opened, DD_ERR_NOT_FOUND if it holds no such entry."""
    c = DdConf()
    check(lib().dd_read_tuned_conf(filename.encode(), device.encode(), nrDMs, C.byref(c)))
    return DedispersionConf.from_c(c)


def writeTunedDedispersionConf(filename: str, device: str, nrDMs: int,
                               conf: DedispersionConf) -> None:
    """Append ``device nrDMs <conf.print()>`` to a tuned-configuration file."""
    c = conf.to_c()
    check(lib().dd_write_tuned_conf(filename.encode(), device.encode(), nrDMs, C.byref(c)))


@dataclass
class KernelEntry:
    """One compiled tile configuration of the engine."""

    index: int
    name: str
    elem_bits: int
    conf: DedispersionConf


DM_STATS = np.dtype([("mean", np.float64), ("stddev", np.float64), ("snr", np.float64),
                     ("peak", np.float32), ("peak_sample", np.uint32)])


def dm_stats(accum, samples: int) -> np.ndarray:
    """Mean, standard deviation, S/N, peak and peak sample of each output row
    from the accumulators :meth:`Plan.run_stats` fills (host array of
    ``rows x 3`` uint64)."""
    acc = np.ascontiguousarray(np.asarray(accum, dtype=np.uint64).reshape(-1, 3))
    out = np.zeros(len(acc), dtype=DM_STATS)
    check(lib().dd_dm_stats_from_accum(acc.ctypes.data_as(C.c_void_p), len(acc), int(samples),
                                       out.ctypes.data_as(C.c_void_p)))
    return out


def kernels() -> list[KernelEntry]:
    """Every compiled tile configuration (the tuner's search space)."""
    out = []
    for i in range(lib().dd_kernel_count()):
        name = C.create_string_buffer(128)
        bits = C.c_uint32(0)
        c = DdConf()
        check(lib().dd_kernel_info(i, name, 128, C.byref(bits), C.byref(c)))
        out.append(KernelEntry(i, name.value.decode(), bits.value, DedispersionConf.from_c(c)))
    return out


def _devptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    raise TypeError(f"expected a device pointer or tensor, got {type(x)!r}")


def _stream(s) -> int:
    if s is None:
        return 0
    if isinstance(s, int):
        return s
    return int(getattr(s, "cuda_stream"))


class Batch:
    """Many single-step problems (1/2/4/8-bit) in one CUDA graph recorded at
    commit(): the problems' own default kernels on concurrent branches, or
    (setPersistent) one persistent direct-tile kernel over all their tiles.
    Device buffers are bound by add()."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(lib().dd_batch_create(C.byref(self._h), device))
        self._keep = []

    def add(self, observation: Observation, inputBits: int, padding: int, shifts, zapped,
            mapping, d_input, d_output, kernel: int | None = None) -> int:
        """Add one problem; `kernel` (a registry index) sets its configuration
        in the graph form (dd_batch_add_with_kernel), else its default."""
        sh = np.ascontiguousarray(shifts, dtype=np.float32)
        z, m = _u32(zapped), _u32(mapping)
        idx = C.c_uint32(0)
        check(lib().dd_batch_add_with_kernel(
            self._h, C.byref(observation.c), inputBits, padding, _ptr(sh, C.c_float),
            _ptr(z, C.c_uint32), _ptr(m, C.c_uint32), C.c_void_p(_devptr(d_input)),
            C.c_void_p(_devptr(d_output)), -1 if kernel is None else int(kernel),
            C.byref(idx)))
        self._keep.append((d_input, d_output))
        return idx.value

    def commit(self) -> None:
        check(lib().dd_batch_commit(self._h))

    def run(self, stream=None, graph: bool = True) -> None:
        check(lib().dd_batch_run(self._h, C.c_void_p(_stream(stream)), int(graph)))

    def check(self, stream=None) -> None:
        check(lib().dd_batch_check(self._h, C.c_void_p(_stream(stream))))

    def info(self) -> dict:
        p, t, g = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().dd_batch_info(self._h, C.byref(p), C.byref(t), C.byref(g)))
        info = {"problems": p.value, "tiles": t.value, "grid": g.value}
        if t.value:
            sh = C.c_int(0)
            check(lib().dd_batch_shared(self._h, C.byref(sh)))
            info["form"] = "graph" if sh.value else "persistent"
        return info

    def setPersistent(self, enable: bool = True) -> None:
        """Commit in the persistent form (one persistent direct-tile kernel)."""
        check(lib().dd_batch_set_persistent(self._h, 1 if enable else 0))

    def close(self) -> None:
        if self._h:
            lib().dd_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """Device-side plan of one mode: tables uploaded once, runs enqueued on a
    stream with device pointers (raw ints or tensors exposing data_ptr())."""

    def __init__(self, observation: Observation, mode: int, inputBits: int, padding: int,
                 conf: DedispersionConf | None = None, device: int = 0,
                 kernel: int | None = None):
        self.observation = observation.copy()
        self.mode, self.inputBits, self.padding = mode, inputBits, padding
        self._h = C.c_void_p()
        if kernel is not None:
            check(lib().dd_plan_create_with_kernel(C.byref(self._h), C.byref(self.observation.c),
                                                   mode, inputBits, padding, kernel, device))
        else:
            cc = conf.to_c() if conf is not None else None
            check(lib().dd_plan_create(C.byref(self._h), C.byref(self.observation.c), mode,
                                       inputBits, padding,
                                       C.byref(cc) if cc is not None else None, device))
        self.layout = layout(self.observation, mode, inputBits if mode != DD_STEP_TWO else 32,
                             padding)

    def setShifts(self, shifts) -> None:
        sh = np.ascontiguousarray(shifts, dtype=np.float32)
        check(lib().dd_plan_set_shifts(self._h, _ptr(sh, C.c_float), sh.size))

    def setZappedChannels(self, zapped) -> None:
        z = _u32(zapped)
        check(lib().dd_plan_set_zapped(self._h, _ptr(z, C.c_uint32), z.size))

    def setBeamMapping(self, mapping) -> None:
        m = _u32(mapping)
        check(lib().dd_plan_set_beam_mapping(self._h, _ptr(m, C.c_uint32), m.size))

    def run(self, d_input, d_output, stream=None) -> None:
        check(lib().dd_plan_run(self._h, C.c_void_p(_devptr(d_input)),
                                C.c_void_p(_devptr(d_output)), C.c_void_p(_stream(stream))))

    def check(self, stream=None) -> None:
        check(lib().dd_plan_check(self._h, C.c_void_p(_stream(stream))))

    def launches(self) -> int:
        n = C.c_uint32(0)
        check(lib().dd_plan_launches(self._h, C.byref(n)))
        return n.value

    def conf(self) -> DedispersionConf:
        c = DdConf()
        check(lib().dd_plan_get_conf(self._h, C.byref(c)))
        return DedispersionConf.from_c(c)

    def run_stats(self, d_input, d_output, d_accum, stream=None) -> None:
        """run() plus detection statistics of the output in ``d_accum`` (device
        buffer of 3 x uint64 per output row: sum, sum of squares, peak key;
        see :func:`dm_stats`)."""
        check(lib().dd_plan_run_stats(self._h, C.c_void_p(_devptr(d_input)),
                                      C.c_void_p(_devptr(d_output)),
                                      C.c_void_p(_devptr(d_accum)),
                                      C.c_void_p(_stream(stream))))

    def setOverlap(self, enable: bool = True) -> None:
        """Launch runs as programmatic dependents of the stream's previous
        kernel (dd_plan_set_overlap): only for consecutive independent runs."""
        check(lib().dd_plan_set_overlap(self._h, 1 if enable else 0))

    def setWaitLimit(self, ns: int) -> None:
        """Limit of each device-side wait for a staged copy, in ns (0: the
        default 2 s); a run whose wait runs out makes check() raise with
        DD_ERR_TIMEOUT (dd_plan_set_wait_limit)."""
        check(lib().dd_plan_set_wait_limit(self._h, int(ns)))

    def adds(self) -> int:
        """Integer adds one run performs (tile padding included)."""
        n = C.c_uint64(0)
        check(lib().dd_plan_adds(self._h, C.byref(n)))
        return n.value

    def close(self) -> None:
        if self._h:
            lib().dd_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self) -> "Plan":
        return self

    def __exit__(self, *exc) -> None:
        self.close()
