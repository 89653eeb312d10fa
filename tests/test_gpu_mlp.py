"""The learned mode's network kernels against the float64 CPU restatement
(tests/mlp_ref.py), training, checkpoints, and the learned mode's equal-error
contract: same hits as the plain solver, fewer Newton iterations."""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import mlp_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = hr.Context(0)
    c.generate_synthetic(6, 6, 6, 5, 5, 0.1, 32, 11)
    c.build_bvh()
    return c


def test_forward_matches_cpu(ctx):
    ctx.mlp_init(3)
    p = ctx.mlp_params()
    rng = np.random.default_rng(0)
    X = rng.normal(size=(1000, 48)).astype(np.float32)
    y = ctx.mlp_forward(X)
    ref = mlp_ref.forward(p, X)
    err = np.abs(y - ref).max() / np.abs(ref).max()
    assert err < 2e-2, err


def test_gradients_match_cpu(ctx):
    ctx.mlp_init(4)
    p = ctx.mlp_params()
    rng = np.random.default_rng(1)
    n = 512
    X = rng.normal(size=(n, 48)).astype(np.float32)
    T = rng.normal(size=(n, 8)).astype(np.float32)
    valid = (rng.uniform(size=n) > 0.1).astype(np.uint8)
    loss, g = ctx.mlp_grad(X, T, valid)
    rloss, rg = mlp_ref.loss_and_grads(p, X, T, valid)
    assert abs(loss - rloss) / rloss < 1e-3
    o = 0
    for i, nn in mlp_ref.DIMS:
        for size in (i * nn, nn):
            a, b = g[o:o + size], rg[o:o + size]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert rel < 3e-2, (o, rel)
            o += size


def test_training_pairs_are_plain_solver_answers(ctx):
    X, T, V = ctx.learn_samples(4096, seed=5)
    assert V.mean() > 0.9
    assert np.isfinite(T[V == 1]).all()
    # entry points lie on the padded box, so xi there is just outside [-1,1]
    assert np.abs(T[V == 1, :3]).max() < 3.0 and np.abs(T[V == 1, :3]).max() > 1.0
    # the same seed gives the same pairs
    X2, T2, V2 = ctx.learn_samples(4096, seed=5)
    assert np.array_equal(X, X2) and np.array_equal(T, T2) and np.array_equal(V, V2)


def test_train_save_load_and_learned_mode(ctx, tmp_path):
    losses = ctx.train_mlp(n_samples=400_000, steps=600, batch=2048, lr=2e-3, seed=9)
    assert losses[-50:].mean() < 0.2 * losses[:20].mean()
    path = str(tmp_path / "net.bin")
    ctx.mlp_save(path)
    p0 = ctx.mlp_params()
    ctx.mlp_load(path)
    assert np.array_equal(p0, ctx.mlp_params())
    cam = hr.Camera((2.5, 2.0, 1.8), (0.5, 0.5, 0.5))
    isos = [-0.3, 0.0, 0.3]
    # the same batched kernels with cold starts are what the network replaces
    ctx.set_mode(hr.MODE_BATCHED)
    _, hp = ctx.render(cam, isos, 256, 192, iso_zero_disables=False, want_rgb=False, want_hits=True)
    sp = ctx.stats()
    ctx.set_mode(hr.MODE_LEARNED)
    _, hl = ctx.render(cam, isos, 256, 192, iso_zero_disables=False, want_rgb=False, want_hits=True)
    sl = ctx.stats()
    ctx.set_mode(hr.MODE_BATCHED)
    same = (hp["kind"] == hl["kind"]) & (hp["elem"] == hl["elem"]) & (hp["face"] == hl["face"])
    print("learned vs batched cold start: id agreement", same.mean(), "newton", sp["newton_iters"], "->", sl["newton_iters"],
          "face", sp["face_iters"], "->", sl["face_iters"], "accepted", sl["mlp_accepted"], "rejected",
          sl["mlp_rejected"])
    assert same.mean() >= 0.995
    # equal error: face hits to the face Newton's tolerance; isosurface hits
    # both meet the reference's stopping rule |u - iso| < 1e-5 (which bounds t
    # only through du/dt, so t itself may differ more where u varies slowly)
    # (face rule: position residual < 1e-4, so t agrees to ~1e-4 / cos(incidence))
    face = same & (hp["kind"] == hr.HIT_FACE)
    dtf = np.abs(hp["t"][face] - hl["t"][face])
    assert (dtf < 2e-4).mean() >= 0.99 and dtf.max() < 2e-3
    isoh = same & (hp["kind"] == hr.HIT_ISO)
    iso_of = np.broadcast_to(np.array(isos, np.float32)[:, None, None], hp.shape)
    for h in (hp, hl):
        assert (np.abs(h["u"][isoh] - iso_of[isoh]) < 2e-5).mean() >= 0.99
    assert np.abs(hp["t"][isoh] - hl["t"][isoh]).max() < 2e-3
    assert sl["newton_iters"] + sl["face_iters"] < 0.7 * (sp["newton_iters"] + sp["face_iters"])
    assert sl["mlp_accepted"] > 4 * sl["mlp_rejected"]
