"""Learned autoregressive proposal (no reference counterpart): gradients of the
hand-written BF16/FP32 training kernels against a torch-CPU FP32 autograd
reference of the same network; log q from the one deterministic kernel in
sampling and scoring mode (bit-identical) and its normalisation; an exact
Metropolis-Hastings chain checked against exact enumeration.

Tolerances: gradients 2e-3 relative to the largest gradient of the layer plus
1e-5 absolute (FP32 accumulation in different orders); torch log q agreement
2e-3 absolute per configuration (the sampling kernel's BF16 hidden activations
restated in torch); normalisation 1e-4."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def learned(pkg):
    import importlib
    return importlib.import_module(pkg.__name__ + ".learned")


def torch_logq(w, D, H, W, cfg, bf16_acts=False, zrow=0):
    """torch FP32 restatement of the network (masks as zeroed 3x3 taps; with
    zrow > 0 layer 0 adds the z-plane tap, the input zrow rows up);
    bf16_acts rounds the hidden activations to BF16 as the tensor-core
    sampling kernel stores them."""
    import torch
    import torch.nn.functional as F
    taps = [(-1, -1), (-1, 0), (-1, 1), (0, -1), (0, 0)]
    x = cfg.view(-1, 1, H, W)
    off = 0
    for l in range(D):
        cin = 1 if l == 0 else 32
        cout = 1 if l == D - 1 else 32
        nt = (5 if zrow else 4) if l == 0 else 5
        n = nt * cin * cout
        wl = w[off:off + n].view(nt, cin, cout)
        off += n
        b = w[off:off + cout]
        off += cout
        grid = [torch.zeros(cout, cin, dtype=w.dtype)] * 9
        for t in range(4 if l == 0 else nt):
            dy, dx = taps[t]
            grid[(1 + dy) * 3 + (1 + dx)] = wl[t].t()
        K = torch.stack(grid, dim=-1).view(cout, cin, 3, 3)
        xin = x
        x = F.conv2d(xin, K, b, padding=1)
        if l == 0 and zrow:
            shifted = F.pad(xin, (0, 0, zrow, 0))[:, :, :H, :]  # input at (y - zrow, x)
            x = x + torch.einsum("bihw,io->bohw", shifted, wl[4])
        if l < D - 1:
            x = torch.relu(x)
            if bf16_acts:
                x = x.to(torch.bfloat16).float()
    logits = x.view(-1, H * W)
    return F.logsigmoid(cfg.view(-1, H * W) * logits).sum(1)


@pytest.mark.parametrize("H,W,D,zrow", [(6, 6, 4, 0), (8, 4, 6, 0), (16, 4, 4, 4)])
def test_gradient_matches_torch_cpu(gpu, H, W, D, zrow):
    """Gradients of the hand-written training kernels against torch-CPU FP32
    autograd of the same network (the last case: the 4^3 raster with layer 0's
    z-plane tap)."""
    import torch
    L = learned(gpu)
    q = L.LearnedProposal(H, W, layers=D, seed=5, zrow=zrow)
    rng = np.random.default_rng(0)
    # perturb biases too so every parameter is exercised
    w0 = q.weights() + rng.normal(0, 0.05, q.n_params).astype(np.float32)
    q.set_weights(w0)
    wq = q.weights()  # BF16-rounded values the kernels use
    cfg = np.where(rng.random((16, H * W)) < 0.5, 1, -1).astype(np.int8)
    g, nll = q.gradient(cfg)
    wt = torch.tensor(wq, dtype=torch.float32, requires_grad=True)
    loss = -torch_logq(wt, D, H, W, torch.tensor(cfg, dtype=torch.float32), zrow=zrow).mean()
    loss.backward()
    gt = wt.grad.numpy()
    assert abs(nll - loss.item()) < 2e-3 * max(1.0, abs(loss.item()))
    scale = np.abs(gt).max()
    assert np.all(np.abs(g - gt) <= 2e-3 * scale + 1e-5), np.abs(g - gt).max() / scale


def test_sample_score_identical_and_matches_torch(gpu):
    import torch
    L = learned(gpu)
    H = W = 8
    q = L.LearnedProposal(H, W, layers=6, seed=9)
    props, lq, lqf = q.sample(64, 3)
    q.sync()
    s1 = q.score(props)
    s2 = q.score(props, flip=True)
    q.sync()
    assert torch.equal(lq, s1) and torch.equal(lqf, s2)
    assert set(torch.unique(props).tolist()) <= {-1, 1}
    ref = torch_logq(torch.tensor(q.weights()), 6, H, W, props.cpu().float(), bf16_acts=True)
    assert torch.max(torch.abs(ref - lq.cpu())) < 2e-3
    # the same step reproduces the same proposals; another step gives others
    p2, l2, _ = q.sample(64, 3)
    p3, _, _ = q.sample(64, 4)
    q.sync()
    assert torch.equal(p2, props) and torch.equal(l2, lq) and not torch.equal(p3, props)


@pytest.mark.parametrize("H,W,D,zrow", [(16, 16, 6, 0), (32, 32, 6, 0), (64, 8, 6, 0),
                                        (12, 20, 4, 0), (64, 8, 6, 8), (144, 12, 5, 12)])
def test_sample_score_identical_at_chain_sizes(gpu, H, W, D, zrow):
    """The sampler and the whole-lattice scorer give bit-identical log q (and
    log q of the negation) at the raster sizes the chains use, 3D rasters with
    layer 0's z-plane tap included."""
    import torch
    L = learned(gpu)
    q = L.LearnedProposal(H, W, layers=D, seed=21, zrow=zrow)
    props, lq, lqf = q.sample(300, 5)
    s1 = q.score(props)
    s2 = q.score(props, flip=True)
    q.sync()
    assert torch.equal(lq, s1) and torch.equal(lqf, s2)
    if zrow:
        ref = torch_logq(torch.tensor(q.weights()), D, H, W, props.cpu().float(),
                         bf16_acts=True, zrow=zrow)
        # FP32 sums of H*W log-sigmoid terms in two different orders: the
        # difference grows with the number of terms (2e-3 at 512 positions)
        tol = 2e-3 * max(1.0, H * W / 512)
        assert torch.max(torch.abs(ref - lq.cpu())) < tol


@pytest.mark.parametrize("H,W,zrow", [(3, 3, 0), (4, 2, 2)])
def test_distribution_is_normalised(gpu, H, W, zrow):
    """q sums to 1 over all configurations (the 2^3 lattice's 4 x 2 raster
    with the z-plane tap too)."""
    import torch
    L = learned(gpu)
    q = L.LearnedProposal(H, W, layers=3, seed=13, zrow=zrow)
    w = q.weights()
    q.set_weights(w * 3.0)  # a sharper, non-trivial distribution
    allc = np.array(list(itertools.product([-1, 1], repeat=H * W)), np.int8)
    d = torch.tensor(allc, device="cuda")
    lq = q.score(d)
    q.sync()
    assert abs(torch.exp(lq.double()).sum().item() - 1.0) < 1e-4


def test_training_reduces_nll(gpu):
    L = learned(gpu)
    data = L.collect_training_set(8, 2, 2.269, chains=32, rounds=16, gap=10, warmup=500)
    q = L.LearnedProposal(8, 8, layers=6, seed=1)
    host = data[:64].cpu().numpy()
    _, nll0 = q.gradient(host)
    q.train(data, batch=64, steps=150, lr=2e-3)
    _, nll1 = q.gradient(host)
    assert nll1 < nll0 - 5.0, (nll0, nll1)


@pytest.mark.parametrize("L_,dim,T", [(4, 2, 2.269), (2, 3, 4.0)])
def test_chain_is_exact(gpu, oracle, L_, dim, T):
    """The learned chain (trained briefly, so proposals are imperfect and
    fallback sweeps interleave) reproduces exact-enumeration E and |M|."""
    import torch
    L = learned(gpu)
    n = L_ ** dim
    H, W = (L_, L_) if dim == 2 else (L_ * L_, L_)
    data = L.collect_training_set(L_, dim, T, chains=32, rounds=16, gap=5, warmup=200)
    q = L.LearnedProposal(H, W, layers=4, seed=2, zrow=L_ if dim == 3 else 0)
    q.train(data, batch=64, steps=60, lr=3e-3)
    ch = L.LearnedChain(q, L_, dim, T, K=2048, sweeps=1, fallback_sweeps=5, min_accept=0.05)
    request_close = ch.close
    ch.start(50)
    es, ms = [], []
    for b in range(40):
        ch.batch()
    # the samples after burn-in, when the sweeps per batch are frozen
    m = ch.m_series()[ch.burn_in * ch.K:]
    e = ch.e_series()[ch.burn_in * ch.K:]
    ex = oracle.exact_enumeration(L_, dim, [T])[0]
    assert abs(m.mean() - ex["M"]) < 0.02, (m.mean(), ex["M"])
    assert abs(e.mean() - ex["E"]) < 0.03, (e.mean(), ex["E"])
    assert np.mean(ch.batch_accept) > 0.05
    request_close()


def test_trained_network_gains_over_untrained(gpu):
    """What the trained network gains: at Tc on 2D L=8 the trained proposal is
    accepted far more often than the same network untrained, and its chain
    decorrelates |M| faster per proposal."""
    L = learned(gpu)
    data = L.collect_training_set(8, 2, 2.269, chains=64, rounds=32, gap=10, warmup=500)
    rates = {}
    for trained in (False, True):
        q = L.LearnedProposal(8, 8, layers=6, seed=4)
        if trained:
            q.train(data, batch=128, steps=300, lr=2e-3)
        ch = L.LearnedChain(q, 8, 2, 2.269, K=2048, sweeps=0, fallback_sweeps=0, min_accept=0.0)
        ch.start(200)
        for _ in range(6):
            ch.batch()
        rates[trained] = float(np.mean(ch.batch_accept))
        ch.close()
    assert rates[True] > 0.05 and rates[True] > 5 * rates[False], rates


def test_long_chain_matches_plain_sampler(gpu):
    """Exactness where the proposal is far from perfect: on 2D L = 8 at T_c the
    briefly trained chain (IMH + one sweep per batch, 600k proposals) and 64
    independent plain Metropolis chains agree on <|m|> and <e> within 4.5
    combined standard errors (the chain's from 20 block means, which include
    its long sticky stretches)."""
    import torch
    L = learned(gpu)
    Ls, T = 8, 2.269
    n = Ls * Ls
    stream = L.TrainingStream(Ls, 2, T, chains=128, gap=10, warmup=1000)
    q = L.LearnedProposal(Ls, Ls, layers=6, seed=5)
    for _ in range(60):
        q.train(stream.next(), batch=128, steps=4, lr=2e-3)
    stream.close()
    ch = L.LearnedChain(q, Ls, 2, T, K=2048, sweeps=1, fallback_sweeps=20, min_accept=0.002)
    ch.start(1000)
    for _ in range(300):
        ch.batch()
    m, e = ch.m_series(), ch.e_series()
    assert np.mean(ch.batch_accept) > 0.02
    ch.close()

    ref = gpu.IsingBatch([Ls], 64, seed=9, dim=2)
    ref.set_temperatures([T] * 64)
    ref.step(2000)
    rb, rm = ref.run_schedule(None, 40000, measure_every=10)
    ref.close()
    rmag = np.abs(rm).astype(float) / n
    ren = -rb.astype(float) / n

    def block_err(x, nb=20):
        B = len(x) // nb
        return x[:B * nb].reshape(nb, B).mean(1).std(ddof=1) / np.sqrt(nb)

    for name, a, r in (("|m|", m, rmag), ("e", e, ren)):
        ea = block_err(a)
        er = r.mean(0).std(ddof=1) / np.sqrt(r.shape[1])
        diff = a.mean() - r.mean()
        assert abs(diff) < 4.5 * np.hypot(ea, er), (name, a.mean(), ea, r.mean(), er)


def test_batch_quantum_is_whole_waves(gpu):
    import torch
    L = learned(gpu)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for H, W in ((16, 16), (32, 32)):
        q = L.LearnedProposal(H, W, layers=6, seed=1)
        k = q.batch_quantum()
        assert k % (16 * sms) == 0 and k >= 16 * sms, (H, W, k, sms)
