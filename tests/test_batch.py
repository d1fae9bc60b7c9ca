"""Batches: uneven beams of mixed input widths in one CUDA graph launch give,
beam by beam, exactly the plain path's output, both in the graph form (each
beam's own default kernel on concurrent branches, shared or direct tile) and
in the persistent form (one persistent direct-tile kernel); beams are also
checked against the CPU oracle."""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

SHAPES = [
    dict(channels=200, bandwidth=1.5, samples=1300, dms=70, dm_step=0.35, bits=8, seed=1),
    dict(channels=96, bandwidth=3.125, samples=700, dms=33, dm_step=0.5, bits=4, seed=2),
    dict(channels=300, bandwidth=1.0, samples=2048, dms=128, dm_step=0.1, bits=2, seed=3),
    dict(channels=64, bandwidth=4.6875, samples=512, dms=32, dm_step=0.25, bits=8, seed=4),
    dict(channels=128, bandwidth=2.34375, samples=999, dms=17, dm_step=0.45, bits=1, seed=5),
]


def build(torch, padding=64, shapes=SHAPES):
    beams = []
    for sh in shapes:
        obs = sh["obs"] if "obs" in sh else syn.shape_observation(sh, padding)
        shifts = dd.getShifts(obs, padding)
        zapped = syn.zapped_mask(sh["channels"], 0.1, sh["seed"], padding)
        mapping = syn.identity_mapping(obs, padding)
        d_in = syn.device_uniform_input(torch, obs, sh["bits"], padding, sh["seed"])
        lay = dd.layout(obs, dd.DD_SINGLE_STEP, sh["bits"], padding)
        d_out = torch.full((lay.output_bytes // 4,), -1.0, device="cuda")
        beams.append((sh, obs, shifts, zapped, mapping, d_in, d_out, lay))
    return beams


def _equals_plain(batch, beams, padding):
    torch = pytest.importorskip("torch")
    for graph in (True, True, False):  # two graph replays, then a direct launch
        for b in beams:
            b[6].fill_(-1.0)
        batch.run(graph=graph)
        batch.check()
        for sh, obs, shifts, zapped, mapping, d_in, d_out, lay in beams:
            plan = dd.Plan(obs, dd.DD_SINGLE_STEP, sh["bits"], padding)
            plan.setShifts(shifts)
            plan.setZappedChannels(zapped)
            plan.setBeamMapping(mapping)
            want = torch.zeros_like(d_out)
            plan.run(d_in, want)
            plan.check()
            plan.close()
            S = obs.getNrSamplesPerBatch()
            rows = lay.output_bytes // 4 // lay.output_row_elems
            g = d_out.view(rows, -1)[:, :S]
            w = want.view(rows, -1)[:, :S]
            assert torch.equal(g, w), sh


def test_batch_matches_plain_path(gpu, oracle):
    torch = pytest.importorskip("torch")
    padding = 64
    beams = build(torch, padding)
    batch = dd.Batch()
    for sh, obs, shifts, zapped, mapping, d_in, d_out, lay in beams:
        batch.add(obs, sh["bits"], padding, shifts, zapped, mapping, d_in, d_out)
    batch.commit()
    info = batch.info()
    assert info["problems"] == len(SHAPES) and info["tiles"] > 0
    assert info["form"] == "graph" and 1 <= info["grid"] <= len(SHAPES)
    _equals_plain(batch, beams, padding)
    # one beam against the CPU oracle
    sh, obs, shifts, zapped, mapping, d_in, d_out, lay = beams[1]
    ref = np.zeros(lay.output_bytes // 4, np.float32)
    oracle.dedispersion(obs.c, zapped, mapping, d_in.cpu().numpy(), ref, shifts, padding,
                        sh["bits"])
    S = obs.getNrSamplesPerBatch()
    got = d_out.cpu().numpy().reshape(-1, lay.output_row_elems)[:, :S]
    np.testing.assert_array_equal(got, ref.reshape(-1, lay.output_row_elems)[:, :S])
    batch.close()


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_mixed_tiles_and_persistent_form(gpu, oracle, persistent):
    """A beam whose partial sums do not fit the shared tile (1 MHz channels
    from 300 MHz, DM step 0.12: ~34 samples more delay per DM step in the
    lowest channel) runs its direct tile beside the others' shared tiles in
    the graph form; the persistent form runs every beam on the persistent
    direct-tile kernel."""
    torch = pytest.importorskip("torch")
    padding = 64
    wide = dict(obs=syn.make_observation(128, 300.0, 1.0, 81.92e-6, 512, 64, 0.0, 0.12,
                                         padding=padding), channels=128, bits=8, seed=9)
    beams = build(torch, padding, SHAPES[:3] + [wide])
    batch = dd.Batch()
    if persistent:
        batch.setPersistent(True)
    for sh, obs, shifts, zapped, mapping, d_in, d_out, lay in beams:
        batch.add(obs, sh["bits"], padding, shifts, zapped, mapping, d_in, d_out)
    batch.commit()
    info = batch.info()
    assert info["form"] == ("persistent" if persistent else "graph")
    assert info["grid"] > 0 and info["problems"] == 4
    _equals_plain(batch, beams, padding)
    # the wide beam (a default plan falls back to a smaller direct tile) against the oracle
    sh, obs, shifts, zapped, mapping, d_in, d_out, lay = beams[3]
    ref = np.zeros(lay.output_bytes // 4, np.float32)
    oracle.dedispersion(obs.c, zapped, mapping, d_in.cpu().numpy(), ref, shifts, padding, 8)
    S = obs.getNrSamplesPerBatch()
    got = d_out.cpu().numpy().reshape(-1, lay.output_row_elems)[:, :S]
    np.testing.assert_array_equal(got, ref.reshape(-1, lay.output_row_elems)[:, :S])
    batch.close()


def test_batch_of_many_small_beams(gpu):
    """200 small beams (more than any fixed parameter space would hold) in
    one graph: every beam equals its plain run."""
    torch = pytest.importorskip("torch")
    padding = 64
    rng = np.random.default_rng(5)
    shapes = [dict(channels=int(rng.choice([32, 64, 96])), bandwidth=2.0,
                   samples=int(rng.integers(64, 512)), dms=int(rng.integers(1, 24)),
                   dm_step=float(rng.uniform(0.1, 0.5)), bits=int(rng.choice([2, 4, 8])),
                   seed=1000 + i) for i in range(200)]
    beams = build(torch, padding, shapes)
    batch = dd.Batch()
    for sh, obs, shifts, zapped, mapping, d_in, d_out, lay in beams:
        batch.add(obs, sh["bits"], padding, shifts, zapped, mapping, d_in, d_out)
    batch.commit()
    assert batch.info()["problems"] == 200 and batch.info()["form"] == "graph"
    _equals_plain(batch, beams, padding)
    batch.close()


def test_batch_with_chosen_configurations(gpu, oracle):
    """Per-beam configurations chosen by the caller (dd_batch_add_with_kernel:
    a tuner's picks) give each beam exactly its plain output; a configuration
    that cannot run a beam is refused and adds nothing."""
    torch = pytest.importorskip("torch")
    padding = 64
    beams = build(torch, padding)
    names = ["swar8_i4_d4_w16_c16_vkUnpackPermuteMad", "shared8_i8_d2_w16",
             "swar8_i2_d8_w8_c16_vkUnpackPermuteMad", "shared8_i4_d2_w16",
             "swar8_i4_d4_w8_c16_vkUnpackPermuteMad"]
    index = {k.name: k.index for k in dd.kernels()}
    batch = dd.Batch()
    for b, name in zip(beams, names):
        sh, obs, shifts, zapped, mapping, d_in, d_out, lay = b
        batch.add(obs, sh["bits"], padding, shifts, zapped, mapping, d_in, d_out,
                  kernel=index[name])
    batch.commit()
    assert batch.info()["form"] == "graph"
    _equals_plain(batch, beams, padding)
    # a 16-bit tile cannot run an 8-bit beam
    sh, obs, shifts, zapped, mapping, d_in, d_out, lay = beams[0]
    with pytest.raises(dd.DedispersionError):
        batch.add(obs, sh["bits"], padding, shifts, zapped, mapping, d_in, d_out,
                  kernel=index["scalar16_i8_d4_w8_c16"])
    assert batch.info()["problems"] == len(beams)
    batch.close()
