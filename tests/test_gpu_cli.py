"""The `analisi -g/-F` command line on the GPU engine: its printed block
averages equal, character for character, what the reference's CLI branch
computes (analisi/main.cpp:552-584 with BlockAverage/MediaVar), rebuilt here
from the oracle's exact per-block buffers.  The reference's own CLI goldens
(tests/data/cli/pair_corr_*) need an input file that is not available."""
import os
import subprocess

import numpy as np
import pytest

import lammps_writer

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "analisi_gb300", "_build", "analisi")


def expected_output(oracle_mod, pos_int, boxes_int, tids, ntypes, rmin, rmax, nbin, tmax,
                    nthreads, skip, every, B, tric):
    T = pos_int.shape[0]
    n_extra = T // (B + 1) + 1
    if not (n_extra < tmax or tmax == 0):
        n_extra = tmax
    s = (T - n_extra) // B
    leff = s if (s < tmax or tmax == 0) else tmax
    nch = ntypes * (ntypes + 1)
    mean = np.zeros((leff, nch, nbin))
    var = np.zeros_like(mean)
    for ib in range(B):
        c = oracle_mod.gofrt_counts(pos_int, boxes_int, tids, ntypes, rmin, rmax, nbin, tmax,
                                    nthreads, skip, every, s, ib * s, tric=tric, per_thread=True)
        calc = oracle_mod.fold_buffer(c, oracle_mod.incr(s, skip))
        delta = calc - mean
        tmp = delta / (ib + 1)
        mean = mean + tmp
        tmp = calc - mean
        tmp = tmp * delta
        var = var + tmp
    var = var / ((B - 1) * B)
    lines = []
    for t in range(0, leff, every):
        for r in range(nbin):
            row = [str(t), str(r)]
            for ch in range(nch):
                row += [f"{mean[t, ch, r]:g}", f"{var[t, ch, r]:g}"]
            lines.append(" ".join(row))
        lines += ["", ""]
    return lines


@pytest.mark.parametrize("tric", [False, True])
def test_cli_matches_reference_block_average(built_engine, oracle_mod, tmp_path, tric):
    from analisi_gb300 import build, workloads
    build.build_host()
    rng = np.random.default_rng(77 + tric)
    T, N, L = 60, 150, 12.0
    pos = np.cumsum(np.concatenate([rng.uniform(0, L, (1, N, 3)),
                                    rng.normal(0, 0.2, (T - 1, N, 3))]), axis=0)
    types = rng.choice([3, 8], N).astype(np.int32)
    row = [0, L, 0, L, 0, L] + ([0.2 * L, 0.1 * L, 0.15 * L] if tric else [])
    boxes = np.tile(row, (T, 1)).astype(float)
    path = str(tmp_path / "traj.bin")
    lammps_writer.write(path, pos, types, boxes, triclinic=tric, nchunk=2)
    nbin, rmin, rmax, tmax, skip, every, nth, B = 40, 0.0, 4.0, 5, 2, 1, 3, 6
    out = subprocess.run([CLI, "-i", path, "-g", str(nbin), "-F", str(rmin), str(rmax), "-S",
                          str(tmax), "-s", str(skip), "-e", str(every), "-N", str(nth), "-B",
                          str(B)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    text = out.stdout.split("\n")
    header = [l for l in text if l.startswith("#")]
    assert header[0].startswith("# The first column is the time difference")
    body = [l for l in text if not l.startswith("#")]
    boxes_int = workloads.lammps_to_internal(boxes)
    pos_int = oracle_mod.pbc_wrap(pos, boxes_int, tric)
    tids, nt = workloads.dense_type_ids(types)
    want = expected_output(oracle_mod, pos_int, boxes_int, tids, nt, rmin, rmax, nbin, tmax, nth,
                           skip, every, B, tric)
    assert body[:len(want)] == want


@pytest.mark.parametrize("flag", ["-q", "-Q", "--mean-square-displacement-self"])
def test_cli_msd_matches_reference_block_average(built_engine, oracle_mod, tmp_path, flag):
    """`analisi -q/-Q/--mean-square-displacement-self`: block averages of MSD as
    analisi/main.cpp:520-551 prints them (mean and variance per type, and per
    type's centre of mass with -Q), against the oracle's running means fed to
    the same MediaVar recurrence; printed with 6 significant digits."""
    from analisi_gb300 import build, workloads
    build.build_host()
    rng = np.random.default_rng(91)
    T, N, L = 50, 120, 10.0
    pos = np.cumsum(np.concatenate([rng.uniform(0, L, (1, N, 3)),
                                    rng.normal(0, 0.3, (T - 1, N, 3))]), axis=0)
    types = rng.choice([2, 6, 4], N).astype(np.int32)
    boxes = np.tile([0, L, 0, L, 0, L], (T, 1)).astype(float)
    path = str(tmp_path / "traj.bin")
    lammps_writer.write(path, pos, types, boxes, triclinic=False, nchunk=3)
    tmax, skip, nth, B = 6, 2, 2, 5
    out = subprocess.run([CLI, "-i", path, flag, "-S", str(tmax), "-s", str(skip), "-N", str(nth),
                          "-B", str(B)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    got = np.array([[float(v) for v in l.split()] for l in out.stdout.strip().split("\n")])
    cm_msd, cm_self = flag == "-Q", flag == "--mean-square-displacement-self"
    tids, nt = workloads.dense_type_ids(types)
    cm = oracle_mod.centres(pos, tids, nt)
    n_extra = T // (B + 1) + 1
    if not (n_extra < tmax or tmax == 0):
        n_extra = tmax
    s = (T - n_extra) // B
    mean = var = None
    for ib in range(B):
        calc = oracle_mod.msd(pos, tids, nt, skip, tmax, s, ib * s, cm_msd, cm_self, cm=cm)
        if mean is None:
            mean, var = np.zeros_like(calc), np.zeros_like(calc)
        delta = calc - mean
        mean = mean + delta / (ib + 1)
        var = var + (calc - mean) * delta
    var = var / ((B - 1) * B)
    want = np.stack([mean.reshape(mean.shape[0], -1), var.reshape(var.shape[0], -1)],
                    axis=-1).reshape(mean.shape[0], -1)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=1e-12)
