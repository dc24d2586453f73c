"""The oracle's path tracers against the reference's own estimators.

The reference's path tracers seed a fresh mt19937_64 from the system clock in
every recursive call (src/pray.cpp:331,357), so their outputs cannot be
reproduced; tests/golden/pt_moments.npz holds per-pixel means and variances of
the reference's unclamped evaluatePathRecursive (src/pray.cpp:342-364) and
evaluatePathRecursiveDiffuse (src/pray.cpp:315-340), run many times per pixel
on a closed room and on the reference's examples/pt_cornell scene
(make_pt_moments.py). Here the oracle's restatements, driven by PCG32 streams,
must have the same expectation per pixel within sampling error
(golden_util.same_expectation: every |z| < 6, mean z^2 in [0.6, 1.3], image
means within 4.5 standard errors):

* Kajiya mode (the reference's recursion) against evaluatePathRecursive;
* branching mode against evaluatePathRecursiveDiffuse;
* the next-event-estimation mode with Russian roulette, which has no
  reference counterpart, against evaluatePathRecursive: the same light
  transport up to the same path depth, so the same expectation when the
  light sampling and the roulette weights are unbiased. This runs on the two
  rooms, whose emitter is a quad apart from every lit surface. It does not
  run on the Cornell scene: the reference's loader marks its whole ceiling as
  emitting (the MTL line "Ke 0     0    0", read the way the vendored
  tinyobjloader reads it), so wall points next to the ceiling see an emitter
  at vanishing distance, the area-sampled 1/d^2 term has no usable variance
  there, and a z-test of a few thousand samples is not valid (the sample
  means fall short of the expectation at a handful of edge pixels).

A planted mistake (the oracle's albedos scaled by 0.98, i.e. an estimator
biased by 2 % or more) must be caught by the same comparison. The CUDA path
tracer equals the oracle within 1e-4 per pixel on identical PCG streams
(test_pt_gpu.py), and test_pt_stats_gpu.py compares it with these fixtures
directly.
"""
import numpy as np
import pytest

from golden import make_pt_moments as M
from golden_util import batch_moments, pt_moments_fixture, same_expectation

KAJIYA, NEE, DIFFUSE = 0, 1, 2


@pytest.fixture(scope="module")
def fx():
    return pt_moments_fixture()


def oracle_estimate(O, mesh, st, mode, depth, spp_total, batches, seed, branching=1, rr=3):
    """Per-pixel mean and variance of the mean of the oracle's estimator:
    `batches` frames of spp_total / batches samples (Kajiya / NEE), or
    spp_total single trees (branching mode), on disjoint PCG streams."""
    orc = O.OracleScene.from_setup(mesh, st)
    frames = []
    if mode == DIFFUSE:
        for k in range(spp_total):
            frames.append(orc.render_pt(st, spp=branching, max_depth=depth, seed=seed, mode=DIFFUSE,
                                        sample_offset=k)[1])
    else:
        per = spp_total // batches
        for b in range(batches):
            frames.append(orc.render_pt(st, spp=per, max_depth=depth, seed=seed, mode=mode, rr_depth=rr,
                                        sample_offset=b * per)[1])
    return batch_moments(frames)


def reference(fx, name):
    runs = int(fx[f"{name}_runs"])
    return fx[f"{name}_mean"], fx[f"{name}_var"] / runs


@pytest.mark.parametrize("name,mode,spp", [
    ("room_kajiya8", KAJIYA, 4096),
    ("rroom3_kajiya6", KAJIYA, 4096),
    ("cornell_kajiya4", KAJIYA, 8192),
    ("room_kajiya8", NEE, 2048),
    ("rroom3_kajiya6", NEE, 2048),
])
def test_oracle_matches_reference_estimator(oracle, fx, name, mode, spp):
    mesh, st = M.case_scene(name)
    depth = M.CASES[name][3]
    m, v = oracle_estimate(oracle, mesh, st, mode, depth, spp, 16, seed=101 + mode)
    rm, rv = reference(fx, name)
    ok, desc = same_expectation(m, v, rm, rv)
    assert ok, f"{name} mode {mode}: {desc}"


@pytest.mark.parametrize("name", ["room_diffuse2", "cornell_diffuse1"])
def test_oracle_branching_matches_reference_estimator(oracle, fx, name):
    mesh, st = M.case_scene(name)
    _, _, _, depth, _, branching, _ = M.CASES[name]
    m, v = oracle_estimate(oracle, mesh, st, DIFFUSE, depth, 512, 0, seed=77, branching=branching)
    rm, rv = reference(fx, name)
    ok, desc = same_expectation(m, v, rm, rv)
    assert ok, f"{name}: {desc}"


def test_planted_albedo_bias_is_caught(oracle, fx):
    """Power check: the same comparison rejects an oracle whose albedos are 2 %
    too dark (planted in the oracle's input on the CPU)."""
    name = "room_kajiya8"
    mesh, st = M.case_scene(name)
    mesh.colors = np.where(mesh.emit[:, None] != 0, mesh.colors, mesh.colors * np.float32(0.98)).astype(np.float32)
    m, v = oracle_estimate(oracle, mesh, st, KAJIYA, M.CASES[name][3], 4096, 16, seed=5)
    rm, rv = reference(fx, name)
    ok, desc = same_expectation(m, v, rm, rv)
    assert not ok, f"a 2 % albedo bias went undetected: {desc}"
