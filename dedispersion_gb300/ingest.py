"""SIGPROC filterbank and PSRDADA input (the role of AstroData's readers in
the reference).

    fb = Filterbank("beam.fil")         # or Dada("beam.dada")
    fb.observation(obs)                 # channels, frequencies, sampling time
    block = fb.read(start, count)       # [count][nchans] uint8, time-major
    fb.to_rows(d_block, d_input, row_bytes, offset)   # device transpose

The headers are parsed and the samples are read by the library
(``dd_filterbank_*``, ``dd_dada_*``); ``to_rows`` transposes a time-major
device block into a plan's channel rows on the GPU, reversing the channel
order for files whose frequencies descend (``foff < 0``, ``BW < 0``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import check, lib
from . import Observation


class FilterbankInfo(C.Structure):
    _fields_ = [("nchans", C.c_uint32), ("nbits", C.c_uint32), ("nifs", C.c_uint32),
                ("nbeams", C.c_uint32), ("ibeam", C.c_uint32), ("data_type", C.c_uint32),
                ("nsamples", C.c_uint64), ("header_bytes", C.c_uint64), ("tsamp", C.c_double),
                ("fch1", C.c_double), ("foff", C.c_double), ("tstart", C.c_double),
                ("refdm", C.c_double), ("source_name", C.c_char * 80)]


class DadaInfo(C.Structure):
    _fields_ = [("nchan", C.c_uint32), ("nbit", C.c_uint32), ("npol", C.c_uint32),
                ("ndim", C.c_uint32), ("nsamples", C.c_uint64), ("header_bytes", C.c_uint64),
                ("obs_offset", C.c_uint64), ("tsamp", C.c_double), ("freq", C.c_double),
                ("bw", C.c_double), ("source", C.c_char * 64), ("utc_start", C.c_char * 32)]


class _TimeMajorFile:
    """Reads and device transpose shared by the two formats."""

    nchans: int
    nbits: int

    def read(self, start: int, count: int) -> np.ndarray:
        """Samples [start, start + count), time-major ([count][nchans] for
        8-bit files; raw bytes otherwise)."""
        nbytes = count * self.nchans * self.nbits // 8
        buf = np.empty(nbytes, dtype=np.uint8)
        self._read(int(start), int(count), buf.ctypes.data_as(C.c_void_p))
        if self.nbits == 8:
            return buf.reshape(count, self.nchans)
        return buf

    @property
    def nsamples(self) -> int:
        return int(self.info.nsamples)

    def read_into(self, start: int, out: np.ndarray) -> int:
        """Read time samples from ``start`` into ``out`` (a contiguous 8-bit
        [count][nchans] array, e.g. a stream's pinned staging): as many as the
        file holds, the rest of ``out`` zero.  Returns the samples read."""
        if self.nbits != 8:
            raise ValueError("read_into takes 8-bit files")
        if out.dtype != np.uint8 or not out.flags.c_contiguous or out.size % self.nchans:
            raise ValueError("out must be a contiguous uint8 [count][nchans] array")
        count = out.size // self.nchans
        have = max(0, min(count, self.nsamples - int(start)))
        if have:
            self._read(int(start), have, C.c_void_p(out.ctypes.data))
        if have < count:
            out.reshape(count, self.nchans)[have:] = 0
        return have

    def to_rows(self, d_block, d_rows, row_bytes: int, offset: int = 0, stream=None) -> None:
        """Device: time-major 8-bit block -> channel rows at sample ``offset``."""
        from . import _devptr, _stream
        if self.nbits != 8:
            raise ValueError("the device transpose takes 8-bit samples")
        count = int(d_block.numel()) // self.nchans if hasattr(d_block, "numel") else None
        if count is None:
            raise TypeError("d_block must be a device tensor")
        check(lib().dd_transpose_time_major(C.c_void_p(_devptr(d_block)), count,
                                            self.nchans, 1 if self.reversed else 0,
                                            C.c_void_p(_devptr(d_rows)), int(row_bytes),
                                            int(offset), C.c_void_p(_stream(stream))))


class Filterbank(_TimeMajorFile):
    """A SIGPROC filterbank file (IF 0 of multi-IF files)."""

    def __init__(self, path: str) -> None:
        self.path = str(path)
        self.info = FilterbankInfo()
        check(lib().dd_filterbank_info_read(self.path.encode(), C.byref(self.info)))
        self.nchans, self.nbits = self.info.nchans, self.info.nbits

    @property
    def reversed(self) -> bool:
        """File channel 0 is the highest frequency (rows are filled reversed)."""
        return self.info.foff < 0

    def observation(self, obs: Observation) -> Observation:
        """Set obs's channels, lowest frequency, bandwidth and sampling time."""
        check(lib().dd_filterbank_observation(C.byref(self.info), C.byref(obs.c)))
        return obs

    def _read(self, start, count, ptr) -> None:
        check(lib().dd_filterbank_read(self.path.encode(), C.byref(self.info), start, count, ptr))


class Dada(_TimeMajorFile):
    """A PSRDADA file of detected, time-major filterbank data."""

    def __init__(self, path: str) -> None:
        self.path = str(path)
        self.info = DadaInfo()
        check(lib().dd_dada_info_read(self.path.encode(), C.byref(self.info)))
        self.nchans, self.nbits = self.info.nchan, self.info.nbit

    @property
    def reversed(self) -> bool:
        """BW < 0: file channel 0 is the highest frequency."""
        return self.info.bw < 0

    def observation(self, obs: Observation) -> Observation:
        check(lib().dd_dada_observation(C.byref(self.info), C.byref(obs.c)))
        return obs

    def _read(self, start, count, ptr) -> None:
        check(lib().dd_dada_read(self.path.encode(), C.byref(self.info), start, count, ptr))


def write_dada(path: str, data: np.ndarray, *, freq: float, bw: float, tsamp_us: float,
               hdr_size: int = 4096, source: str = "synthetic", extra: dict | None = None) -> None:
    """Write a PSRDADA file: data is time-major [samples][nchan] uint8 (file
    channel order).  For tests and examples."""
    data = np.ascontiguousarray(data, dtype=np.uint8)
    keys = {"HDR_VERSION": "1.0", "HDR_SIZE": str(hdr_size), "NCHAN": str(data.shape[1]),
            "NBIT": "8", "NPOL": "1", "NDIM": "1", "ORDER": "TF", "TSAMP": repr(tsamp_us),
            "FREQ": repr(freq), "BW": repr(bw), "SOURCE": source,
            "UTC_START": "2026-01-01-00:00:00", "OBS_OFFSET": "0"}
    keys.update(extra or {})
    text = "".join(f"{k:<16}{v}\n" for k, v in keys.items()).encode()
    if len(text) > hdr_size:
        raise ValueError("header does not fit HDR_SIZE")
    with open(path, "wb") as f:
        f.write(text + b"\0" * (hdr_size - len(text)))
        f.write(data.tobytes())


def write_filterbank(path: str, data: np.ndarray, *, fch1: float, foff: float, tsamp: float,
                     tstart: float = 60000.0, source_name: str = "synthetic") -> None:
    """Write a SIGPROC filterbank file: data is time-major [samples][nchans]
    uint8 (file channel order).  For tests and examples."""
    def s(x: str) -> bytes:
        b = x.encode()
        return np.int32(len(b)).tobytes() + b

    def i(k: str, v: int) -> bytes:
        return s(k) + np.int32(v).tobytes()

    def d(k: str, v: float) -> bytes:
        return s(k) + np.float64(v).tobytes()

    data = np.ascontiguousarray(data, dtype=np.uint8)
    hdr = (s("HEADER_START") + i("telescope_id", 0) + i("machine_id", 0) + i("data_type", 1)
           + s("source_name") + s(source_name) + d("fch1", fch1) + d("foff", foff)
           + i("nchans", data.shape[1]) + i("nbits", 8) + d("tstart", tstart) + d("tsamp", tsamp)
           + i("nifs", 1) + s("HEADER_END"))
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(data.tobytes())
