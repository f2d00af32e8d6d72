"""GPU parity of the learned guiding surrogate (csrc/pg_mlp.cu) with its FP64
oracle (oracle/mlp_oracle.py).  The kernels keep weights and activations in
BF16 with FP32 accumulation; the oracle runs in FP64 with the same BF16
weights and BF16-rounded layer inputs, so the loss agrees to 2e-3 and each
layer's gradient to 3e-2 in relative L2 norm (the kernels also round the
backward signals to BF16)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

BOX = np.array([-2.0, -1.0, -1.5, 2.0, 3.0, 1.5], dtype=np.float32)
LOSS_RTOL = 2e-3
GRAD_REL_L2 = 3e-2


def records(workloads, rng, n, invalid=0.05, kappa=20.0):
    """Positions in BOX; directions from a position-dependent vMF around the
    direction to a point light; lognormal weights; a few INVALID records."""
    rec = np.zeros(n, dtype=workloads.RECORD_DTYPE)
    pos = BOX[:3] + (BOX[3:] - BOX[:3]) * rng.random((n, 3))
    mu = np.array([0.5, 4.0, 0.2]) - pos
    mu /= np.linalg.norm(mu, axis=1, keepdims=True)
    # vMF sample around mu (Wood's method in closed form for S^2)
    u = rng.random(n)
    ct = 1.0 + np.log(u + (1.0 - u) * np.exp(-2.0 * kappa)) / kappa
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    ph = 2.0 * np.pi * rng.random(n)
    a = np.where(np.abs(mu[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t1 = np.cross(mu, a)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(mu, t1)
    d = mu * ct[:, None] + t1 * (st * np.cos(ph))[:, None] + t2 * (st * np.sin(ph))[:, None]
    rec["position"] = pos
    rec["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rec["weight"] = rng.lognormal(0.0, 1.0, n)
    rec["pdf"] = 1.0
    rec["flags"] = 0
    rec["flags"][rng.random(n) < invalid] = 0xFFFFFFFF
    return rec


def dev(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1).copy()).cuda()


def oracle_view(theta):
    """The parameters as the kernels use them: BF16 weight matrices, FP32 biases."""
    p = M.unpack(theta.astype(np.float64))
    for k in ("W1", "W2", "W3", "W4"):
        p[k] = M.bf16(p[k])
    return M.pack(p)


def oracle_loss_grad(theta, rec):
    w = np.where(rec["flags"] == 0xFFFFFFFF, 0.0, rec["weight"]).astype(np.float64)
    return M.loss_and_grad(oracle_view(theta), rec["position"].astype(np.float64),
                           rec["direction"].astype(np.float64), w, BOX.astype(np.float64), act_round=M.bf16)


def block_errors(g, want):
    out = {}
    o = 0
    for name, shape in M.SHAPES:
        n = int(np.prod(shape))
        a, b = g[o:o + n], want[o:o + n]
        out[name] = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        o += n
    return out


@pytest.mark.parametrize("n", [1, 63, 3001])
def test_loss_and_gradient_match_oracle(n, cuda, pkg, abi, workloads):
    torch = cuda
    rng = np.random.default_rng(n)
    net = pkg.Surrogate(BOX, batch=4096)
    theta = net.params()
    # move off the initialisation so every layer carries signal
    theta = theta + (0.03 * rng.normal(size=theta.shape)).astype(np.float32) * (theta != 0)
    net.set_params(theta)
    rec = records(workloads, rng, n)
    rec["flags"][0] = 0  # at least one valid record
    grad = torch.zeros(abi.MLP_PARAMS, dtype=torch.float32, device="cuda")
    loss = net.loss_grad(dev(torch, rec), n, grad)
    want_loss, want_grad = oracle_loss_grad(theta, rec)
    assert abs(loss - want_loss) <= LOSS_RTOL * max(1.0, abs(want_loss)), (loss, want_loss)
    errs = block_errors(grad.cpu().numpy().astype(np.float64), want_grad)
    for name in ("W1", "W2", "W3", "W4", "b1", "b2", "b3", "b4"):
        assert errs[name] < GRAD_REL_L2, errs
    net.close()


@pytest.mark.parametrize("n", [1, 200, 3001])
def test_tensor_core_step_equals_warp_mma_step(n, cuda, pkg, abi, workloads):
    """The fused tcgen05 step and the warp-level mma.sync kernels compute the same
    loss and gradient: BF16 operands rounded at the same points, FP32 sums in a
    different order."""
    torch = cuda
    rng = np.random.default_rng(100 + n)
    net = pkg.Surrogate(BOX, batch=4096)
    theta = net.params()
    theta = theta + (0.03 * rng.normal(size=theta.shape)).astype(np.float32) * (theta != 0)
    net.set_params(theta)
    rec = records(workloads, rng, n)
    rec["flags"][0] = 0
    d = dev(torch, rec)
    out = {}
    for path in (abi.PG_MLP_PATH_TCGEN05, abi.PG_MLP_PATH_WARP_MMA):
        net.set_path(path)
        grad = torch.zeros(abi.MLP_PARAMS, dtype=torch.float32, device="cuda")
        loss = net.loss_grad(d, n, grad)
        out[path] = (loss, grad.cpu().numpy().astype(np.float64))
    (la, ga), (lb, gb) = out[abi.PG_MLP_PATH_TCGEN05], out[abi.PG_MLP_PATH_WARP_MMA]
    assert abs(la - lb) <= 1e-5 * max(1.0, abs(lb)), (la, lb)
    errs = block_errors(ga, gb)
    for name in ("W1", "W2", "W3", "W4", "b1", "b2", "b3", "b4"):
        assert errs[name] < 1e-2, errs
    net.close()


def test_tensor_core_inference_equals_warp_mma_inference(cuda, pkg, abi):
    """The tcgen05 forward pass (pg_mlp_infer's default) against the warp-level one:
    the same BF16 roundings, but FP32 sums in another order and the encoding's
    fast sine can move an activation across a BF16 rounding boundary (2^-9
    relative), hence tolerances at that scale."""
    torch = cuda
    rng = np.random.default_rng(17)
    net = pkg.Surrogate(BOX)
    theta = net.params()
    net.set_params(theta + (0.05 * rng.normal(size=theta.shape)).astype(np.float32) * (theta != 0))
    n = 1000
    lo, hi = np.array(BOX[:3]), np.array(BOX[3:])
    pos = torch.from_numpy((lo + (hi - lo) * rng.random((n, 3))).astype(np.float32)).cuda()
    out = {}
    for path in (abi.PG_MLP_PATH_TCGEN05, abi.PG_MLP_PATH_WARP_MMA):
        net.set_path(path)
        mix = torch.zeros(n * 80, dtype=torch.float32, device="cuda")
        net.infer(pos, n, mix)
        torch.cuda.synchronize()
        out[path] = mix.cpu().numpy().reshape(n, 16, 5)
    a, b = out[abi.PG_MLP_PATH_TCGEN05], out[abi.PG_MLP_PATH_WARP_MMA]
    np.testing.assert_allclose(a[:, :, 0], b[:, :, 0], atol=2e-3)
    # unit means: a component with a short raw mean vector turns a BF16-level change
    # into a larger change of direction, so a few elements may move more
    dm = np.abs(a[:, :, 1:4] - b[:, :, 1:4])
    assert (dm > 2e-3).mean() < 1e-3 and dm.max() < 5e-2, (dm.max(), (dm > 2e-3).mean())
    np.testing.assert_allclose(a[:, :, 4], b[:, :, 4], rtol=1e-2)
    net.close()


def test_inference_matches_oracle(cuda, pkg, abi):
    torch = cuda
    rng = np.random.default_rng(5)
    net = pkg.Surrogate(BOX)
    theta = net.params()
    theta = theta + (0.05 * rng.normal(size=theta.shape)).astype(np.float32) * (theta != 0)
    net.set_params(theta)
    n = 777
    pos = (BOX[:3] + (BOX[3:] - BOX[:3]) * rng.random((n, 3))).astype(np.float32)
    out = torch.zeros(n * 80, dtype=torch.float32, device="cuda")
    net.infer(torch.from_numpy(pos).cuda(), n, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(n, 16, 5)
    want = M.mixture(M.forward(oracle_view(theta), M.encode(pos, BOX), act_round=M.bf16)["o"])
    np.testing.assert_allclose(got[:, :, 0].sum(1), 1.0, atol=1e-5)
    np.testing.assert_allclose(got[:, :, 0], want["pi"], atol=3e-3)
    cos = (got[:, :, 1:4] * want["mu"]).sum(-1)
    assert cos.min() > 0.999
    np.testing.assert_allclose(got[:, :, 4], want["kappa"], rtol=2e-2)
    net.close()


def test_first_adam_step_matches_oracle(cuda, pkg, abi, workloads):
    """Adam's first step moves each parameter by lr * g / (|g| + eps) ~ lr *
    sign(g): the signs of the GPU update follow the oracle gradient."""
    torch = cuda
    rng = np.random.default_rng(9)
    n = 2048
    net = pkg.Surrogate(BOX, batch=n, lr=1e-3)
    theta0 = net.params()
    rec = records(workloads, rng, n)
    net.train(dev(torch, rec), n)
    delta = net.params().astype(np.float64) - theta0
    _, g = oracle_loss_grad(theta0, rec)
    big = np.abs(g) > 1e-2 * np.abs(g).max()
    agree = np.sign(delta[big]) == -np.sign(g[big])
    assert agree.mean() > 0.99, agree.mean()
    np.testing.assert_allclose(np.abs(delta[big]), 1e-3, rtol=2e-2)
    net.close()


def test_training_reduces_loss(cuda, pkg, abi, workloads):
    torch = cuda
    rng = np.random.default_rng(11)
    n = 1 << 16
    rec = records(workloads, rng, n, kappa=50.0)
    held = records(workloads, rng, 8192, kappa=50.0)
    net = pkg.Surrogate(BOX, batch=1 << 13, lr=3e-3)
    d_rec, d_held = dev(torch, rec), dev(torch, held)
    l0 = net.loss_grad(d_held, 8192)
    for _ in range(12):
        net.train(d_rec, n)
    l1 = net.loss_grad(d_held, 8192)
    # the held-out NLL falls well below the initial one (a kappa-50 vMF has NLL ~ -1.07)
    assert np.isfinite(l1) and l1 < l0 - 1.5 and l1 < 0.0, (l0, l1)
    net.close()


def test_training_reports_its_batch_loss_bit_for_bit(cuda, pkg, abi, workloads):
    """pg_mlp_train sums each batch's loss partials inside its update kernel (one
    warp, in the pairing order of the separate kernel pg_mlp_loss_grad uses): for a
    one-batch pass the loss it reports equals pg_mlp_loss_grad's on the same
    weights exactly.  40000 records: 313 tiles over every SM's partial."""
    torch = cuda
    rng = np.random.default_rng(23)
    n = 40000
    rec = records(workloads, rng, n, kappa=20.0)
    rec["flags"][0] = 0
    net = pkg.Surrogate(BOX, batch=1 << 16)
    d = dev(torch, rec)
    la = net.loss_grad(d, n)
    lb = net.train(d, n)
    assert np.isfinite(la) and la == lb, (la, lb)
    net.close()


def collect(torch, pkg, abi, G, sc, pg, col, spp_list, seed0, guided_after_first=True):
    """Training passes with recording; returns the valid records of all passes
    (host, bucketed by region per pass)."""
    info = sc.info()
    P = info.camera.width * info.camera.height
    img = torch.zeros(P * 3, dtype=torch.float32, device="cuda")
    out = []
    for i, spp in enumerate(spp_list):
        p = abi.render_params(spp=spp, max_depth=10, seed=seed0 + 1000 * i,
                              use_guiding=1 if (guided_after_first and i > 0) else 0, record_samples=1)
        sc.render(p, img, guide=pg.ctx, records_dev=col.buffer)
        rec, _ = col.get_sorted_data(pg)
        out.append(rec)
        pg.update(col)
    torch.cuda.synchronize()
    return np.concatenate(out)


def test_surrogate_beside_the_fit_lowers_held_out_nll(cuda, pkg, abi):
    """What the network adds to the per-region fit: trained on the same sparse
    records (two short passes), it is judged per region against the fit on a
    second set of records; the regions where it wins take its mixture, and the
    weighted NLL (KL up to a constant) of a third, held-out set falls.  The
    combined guide still renders the same expectation."""
    import __graft_entry__ as entry
    G = entry.load_submodule("guiding")
    torch = cuda
    W, H = 160, 90
    sc = pkg.Scene.cornell(W, H, ico_level=4)
    box = np.array(sc.get_scene_size(), dtype=np.float32)
    pg = G.PathGuiding(12, box)
    col = G.SampleCollector(pg.get_region_count(), W, H)
    train = collect(torch, pkg, abi, G, sc, pg, col, (1, 2), seed0=11)
    net = pkg.Surrogate(box, batch=1 << 13, lr=1e-3)
    d_train = dev(torch, train)
    for _ in range(8):
        net.train(d_train, train.shape[0])
    P = W * H
    img = torch.zeros(P * 3, dtype=torch.float32, device="cuda")

    def records_pass(seed):
        sc.render(abi.render_params(spp=4, max_depth=10, seed=seed, record_samples=1), img, guide=pg.ctx,
                  records_dev=col.buffer)
        rec, _ = col.get_sorted_data(pg)
        return rec

    judge = records_pass(501)
    held = records_pass(777)
    d_held = dev(torch, held)
    nll_fit = pg.ctx.guide_nll(d_held, held.shape[0])
    switched = net.judge_guide(pg.ctx, dev(torch, judge), judge.shape[0], min_records=32)
    nll_comb = pg.ctx.guide_nll(d_held, held.shape[0])
    assert switched > 0
    assert nll_comb < nll_fit - 0.01, (nll_fit, nll_comb, switched)
    # unbiased with the combined guide
    g = torch.zeros(P * 3, dtype=torch.float32, device="cuda")
    sc.render(abi.render_params(spp=512, max_depth=10, seed=3, use_guiding=1), g, guide=pg.ctx)
    p = torch.zeros(P * 3, dtype=torch.float32, device="cuda")
    sc.render(abi.render_params(spp=512, max_depth=10, seed=4), p)
    torch.cuda.synchronize()
    gm, pm = g.mean().item(), p.mean().item()
    assert abs(gm - pm) / pm < 0.02
    net.close()
    pg.close()


def test_network_guide_renders_unbiased(cuda, pkg, abi):
    """pg_mlp_write_guide: the network alone as the guide of a fine region
    grid (no fit) keeps the image's expectation."""
    torch = cuda
    W, H = 96, 54
    sc = pkg.Scene.cornell(W, H, ico_level=3)
    box = np.array(sc.get_scene_size(), dtype=np.float32)
    net = pkg.Surrogate(box)
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=1 << 14)
    ctx.set_regions(14, box)
    net.write_guide(ctx)
    P = W * H
    g = torch.zeros(P * 3, dtype=torch.float32, device="cuda")
    sc.render(abi.render_params(spp=1024, max_depth=10, seed=3, use_guiding=1), g, guide=ctx)
    p = torch.zeros(P * 3, dtype=torch.float32, device="cuda")
    sc.render(abi.render_params(spp=1024, max_depth=10, seed=4), p)
    torch.cuda.synchronize()
    assert np.isfinite(g.cpu().numpy()).all()
    assert abs(g.mean().item() - p.mean().item()) / p.mean().item() < 0.02
    net.close()
    ctx.close()
