"""The CUDA path tracer against the reference's own estimators and against the
oracle at the benchmark's sizes (GPU).

1. Statistical parity with the reference (tests/golden/pt_moments.npz, written
   by make_pt_moments.py from the reference's evaluatePathRecursive,
   src/pray.cpp:342-364, and evaluatePathRecursiveDiffuse, :315-340): the CUDA
   frames' per-pixel expectation must equal the reference estimator's within
   sampling error (golden_util.same_expectation: every |z| < 6, mean z^2 in
   [0.6, 1.3], image means within 4.5 standard errors). Kajiya mode on the
   per-pixel kernel, next-event estimation + Russian roulette on the
   wavefront scheduler (rooms only; the Cornell scene's emitting ceiling is
   explained in test_pt_reference_stats.py), branching mode.
2. The benchmark's closed room (101k triangles, 1024 x 1024, 64 spp, depth 8,
   NEE + RR after depth 3): a band of eight central rows of the full GPU frame
   against the oracle on the same PCG streams, 1e-4 relative per pixel.
3. The 64-scene batch (16 spp, depth 6, Kajiya, sky background): a displaced
   icosphere and a triangle soup from the one persistent launch, a band of
   central rows each against the oracle, 1e-4 relative per pixel.
"""
import numpy as np
import pytest

from golden import make_pt_moments as M
from golden_util import batch_moments, pt_moments_fixture, same_expectation
from nostrum_pray_gb300 import native, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL, ATOL = 1e-4, 1e-6


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    native.lib()


@pytest.fixture(scope="module")
def fx():
    return pt_moments_fixture()


def reference(fx, name):
    return fx[f"{name}_mean"], fx[f"{name}_var"] / int(fx[f"{name}_runs"])


def gpu_estimate(name, mode, frames, spp, scheduler, seed):
    mesh, st = M.case_scene(name)
    _, _, _, depth, _, branching, _ = M.CASES[name]
    sc = native.Scene.from_setup(mesh, st)
    out = []
    for k in range(frames):
        if mode == native.PT_DIFFUSE:
            p = native.pt_params(st, spp=branching, max_depth=depth, seed=seed, mode=mode, sample_offset=k)
        else:
            p = native.pt_params(st, spp=spp, max_depth=depth, seed=seed, mode=mode, rr_depth=3,
                                 scheduler=scheduler, sample_offset=k * spp)
        out.append(sc.render_pt_host(p)[1])
    sc.close()
    return batch_moments(out)


@pytest.mark.parametrize("name,mode,sched", [
    ("room_kajiya8", native.PT_KAJIYA, native.SCHED_PIXEL),
    ("rroom3_kajiya6", native.PT_KAJIYA, native.SCHED_PIXEL),
    ("cornell_kajiya4", native.PT_KAJIYA, native.SCHED_PIXEL),
    ("room_kajiya8", native.PT_NEE, native.SCHED_WAVEFRONT),
    ("rroom3_kajiya6", native.PT_NEE, native.SCHED_WAVEFRONT),
])
def test_gpu_matches_reference_estimator(fx, name, mode, sched):
    m, v = gpu_estimate(name, mode, 16, 4096, sched, seed=900 + mode)
    ok, desc = same_expectation(m, v, *reference(fx, name))
    assert ok, f"{name} mode {mode}: {desc}"


@pytest.mark.parametrize("name", ["room_diffuse2", "cornell_diffuse1"])
def test_gpu_branching_matches_reference_estimator(fx, name):
    m, v = gpu_estimate(name, native.PT_DIFFUSE, 1024, 0, native.SCHED_PIXEL, seed=31)
    ok, desc = same_expectation(m, v, *reference(fx, name))
    assert ok, f"{name}: {desc}"


def band_matches_oracle(oracle, mesh, st, rad, spp, depth, seed, mode, rows):
    r0, r1 = rows
    orc = oracle.OracleScene.from_setup(mesh, st)
    _, orad, _ = orc.render_pt(st, spp=spp, max_depth=depth, seed=seed, mode=mode, rr_depth=3, rows=rows)
    got = rad[r0:r1]
    bad = ~np.isclose(got, orad, rtol=RTOL, atol=ATOL)
    assert int(bad.sum()) == 0, f"{int(bad.sum())} radiance values differ; max abs {np.abs(got - orad).max()}"
    assert float(orad.max()) > 0.0


@pytest.mark.slow
def test_full_room_band_matches_oracle(oracle):
    m = scenes.room()
    st = scenes.room_setup(1024, 1024, spp=64, max_depth=8)
    sc = native.Scene.from_setup(m, st)
    rad = torch.empty((1024, 1024, 3), dtype=torch.float32, device="cuda")
    p = native.pt_params(st, seed=1, mode=native.PT_NEE, rr_depth=3, scheduler=native.SCHED_WAVEFRONT)
    sc.render_pt(p, None, rad)
    torch.cuda.synchronize()
    band_matches_oracle(oracle, m, st, rad.cpu().numpy(), 64, 8, 1, native.PT_NEE, (508, 516))
    sc.close()


@pytest.mark.slow
def test_full_batch_scenes_match_oracle(oracle):
    items = scenes.batch_workload(64, seed=0)
    scs, params, outs = [], [], []
    for i, (mesh, st) in enumerate(items):
        scs.append(native.Scene.from_setup(mesh, st))
        params.append(native.pt_params(st, seed=i, mode=native.PT_KAJIYA))
        outs.append((torch.empty((st.height, st.width, 3), dtype=torch.uint8, device="cuda"),
                     torch.empty((st.height, st.width, 3), dtype=torch.float32, device="cuda")))
    b = native.Batch(scs, params, outs)
    b.tune()
    b.render()
    torch.cuda.synchronize()
    sphere = next(i for i, (m, _) in enumerate(items) if m.n in {20 * 4 ** k for k in range(2, 8)})
    soup = next(i for i, (m, _) in enumerate(items) if m.n not in {20 * 4 ** k for k in range(2, 8)})
    for i in (sphere, soup):
        mesh, st = items[i]
        c = st.height // 2
        band_matches_oracle(oracle, mesh, st, outs[i][1].cpu().numpy(), st.num_samples, st.max_depth_pt, i,
                            native.PT_KAJIYA, (c - 4, c + 4))
