"""The reference's own GPU kernels (the "plain form" baseline, oracle/plain_form.py)
launched on this GPU: they reproduce the reference's CPU results within the
reference's own CPU-vs-GPU tolerance (1e-3 on distance and depth,
examples/main.cpp:184-188), which shows the harness feeds them the reference's
layouts and launch shapes.  The engine is compared with the same FP64 oracle for
contrast.  Skipped where the cubin was not built (it needs the reference sources)."""
import numpy as np
import pytest

from ogx import workloads as W

pytestmark = pytest.mark.gpu


def _plain():
    from oracle import plain_form
    if not plain_form.available():
        pytest.skip("plain-form cubin not built here (needs the reference sources)")
    return plain_form


@pytest.mark.parametrize("gen", ["ellipsoid", "powerlaw"])
def test_plain_form_reproduces_reference_cpu(engine, orc, gen):
    import torch
    pf = _plain()
    b = W.ellipsoid(seed=21, n_pairs=2000) if gen == "ellipsoid" else W.powerlaw(seed=22, n_pairs=2000)
    coords = torch.from_numpy(b.coords).cuda()
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    plain = pf.PlainForm(0).load(coords, b.offsets, b.counts)
    out = plain.run(pairs)
    torch.cuda.synchronize()
    dist = out["dist"].cpu().numpy().astype(np.float64)
    normal = out["normal"].cpu().numpy().astype(np.float64)
    plain.close()
    ref32 = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f32", threads=16)
    o64 = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
    assert np.isfinite(dist).all()
    within = np.abs(dist - ref32["dist"]) <= 1e-3
    assert within.mean() >= 0.99, f"plain form vs reference CPU FP32: {within.mean():.4f} within 1e-3"
    hit = ref32["dist"] < 0
    n_ok = np.linalg.norm(normal[hit] - ref32["normal"][hit], axis=1) <= 1e-3
    assert n_ok.mean() >= 0.95, f"contact normals within 1e-3 of the reference CPU: {n_ok.mean():.4f}"
    # contrast: the reference's FP32 kernels against the FP64 oracle at 1e-5 relative
    scale = np.maximum(1.0, np.abs(o64["dist"]))
    plain_tight = np.mean(np.abs(dist - o64["dist"]) <= 1e-5 * scale)
    ours = engine.query(b, engine.MODE_GJK_EPA)
    ours_tight = np.mean(np.abs(ours["dist"] - o64["dist"]) <= 1e-5 * scale)
    print(f"\n{gen}: distances within 1e-5 of the FP64 oracle: plain form {plain_tight:.4f}, engine {ours_tight:.4f}")
    assert ours_tight >= plain_tight
