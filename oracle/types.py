"""ctypes mirrors of the two structs the oracle's C entry points take
(``dd_observation`` and ``dd_conf`` of include/dedisp_gb300.h) -- TEST
INFRASTRUCTURE ONLY.

The oracle keeps its own copy so that loading it never imports the engine
package (the CPU baseline and the reference arm of the benchmark must run
without the engine's library in the process).  The oracle's entry points take
these structs by address (``c_void_p``), so a caller may pass either this
mirror or the engine's own struct of the same layout;
tests/test_oracle_workload.py checks that the two layouts agree field by
field.
"""
from __future__ import annotations

import ctypes as C


class DdObservation(C.Structure):
    """dd_observation: the AstroData::Observation state the path reads."""

    _fields_ = [
        ("nr_beams", C.c_uint32),
        ("nr_synthesized_beams", C.c_uint32),
        ("nr_channels", C.c_uint32),
        ("nr_subbands", C.c_uint32),
        ("nr_samples_per_batch", C.c_uint32),
        ("nr_samples_per_dispersed_batch", C.c_uint32),
        ("nr_samples_per_batch_subbanding", C.c_uint32),
        ("nr_samples_per_dispersed_batch_subbanding", C.c_uint32),
        ("nr_dms", C.c_uint32),
        ("nr_dms_subbanding", C.c_uint32),
        ("downsampling", C.c_uint32),
        ("nr_zapped_channels", C.c_uint32),
        ("first_dm", C.c_float),
        ("dm_step", C.c_float),
        ("first_dm_subbanding", C.c_float),
        ("dm_step_subbanding", C.c_float),
        ("sampling_time", C.c_float),
        ("min_freq", C.c_float),
        ("channel_bandwidth", C.c_float),
    ]


class DdConf(C.Structure):
    """dd_conf: DedispersionConf's nine fields, in the tuned-file order."""

    _fields_ = [(n, C.c_uint32) for n in (
        "split_batches", "local_mem", "unroll", "threads_d0", "threads_d1", "threads_d2",
        "items_d0", "items_d1", "items_d2")]
