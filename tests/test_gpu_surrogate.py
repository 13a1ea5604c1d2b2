"""GPU: the surrogate's kernels (GEMM layouts, gradients, AdamW) against
FP32/FP64 references, and the trained surrogate against the tracker."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from onekapy_gb300 import _capi as C  # noqa: E402
from onekapy_gb300 import engine as E  # noqa: E402
from onekapy_gb300 import sites as S  # noqa: E402
from onekapy_gb300 import surrogate as SG  # noqa: E402


@pytest.mark.parametrize("flags", [0, 1])
@pytest.mark.parametrize("a_kmajor,b_kmajor", [(True, True), (True, False), (False, True), (False, False)])
@pytest.mark.parametrize("M,N,K,splitk", [(256, 384, 96, 1), (200, 72, 64, 1), (128, 512, 1024, 8),
                                          (296, 520, 512, 1), (64, 65536, 512, 1), (512, 512, 65536, 37)])
def test_gemm_layouts_match_fp32(flags, a_kmajor, b_kmajor, M, N, K, splitk):
    """Both GEMM kernels (tcgen05 where it applies, and the forced mma.sync
    kernel) against an FP32 product of the same BF16 operands."""
    dev = C.device()
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    A = torch.randn((M, K), generator=g).to(dev)
    B = torch.randn((K, N), generator=g).to(dev)
    bias = torch.randn(N, generator=g).to(dev) if splitk == 1 else None
    Ab = (A if a_kmajor else A.T.contiguous()).to(torch.bfloat16).contiguous()
    Bb = (B.T.contiguous() if b_kmajor else B).to(torch.bfloat16).contiguous()
    Cf = torch.zeros((M, N), dtype=torch.float32, device=dev)
    SG.gemm(Ab, a_kmajor, Bb, b_kmajor, Cf, M, N, K, bias=bias, splitk=splitk, flags=flags)
    ref = (Ab.float() if a_kmajor else Ab.float().T) @ (Bb.float().T if b_kmajor else Bb.float())
    if bias is not None:
        ref = ref + bias
    tc = SG.gemm_path(a_kmajor, b_kmajor, K, splitk=splitk, flags=flags)
    assert tc == int(flags == 0 and a_kmajor and b_kmajor and K % 64 == 0)
    assert SG.tc_status() == 0
    assert torch.allclose(Cf, ref, rtol=1e-3, atol=1e-3 * math.sqrt(K)), float((Cf - ref).abs().max())


@pytest.mark.parametrize("M,N,K,splitk,epi", [(512, 4096, 512, 1, "f32"), (384, 768, 128, 1, "f32"),
                                               (512, 1024, 4096, 4, "f32"), (1024, 1536, 512, 1, "gelu"),
                                               (2048, 4096, 512, 1, "sigsum"), (136, 520, 64, 1, "f32")])
def test_tcgen05_cta_pairs_match_single_ctas(M, N, K, splitk, epi):
    """The tcgen05 GEMM in CTA pairs (clusters of two sharing the B slice by
    TMA multicast; taken when M has an even number of 128-row tiles) against
    the same kernel one CTA per tile (flags bit 1): the same accumulation,
    so identical results (split-K adds its slices atomically: within
    rounding), and both against an FP32 product."""
    dev = C.device()
    g = torch.Generator(device="cpu").manual_seed(M + 7 * N + K)
    A = (torch.randn((M, K), generator=g) / math.sqrt(K)).to(dev).to(torch.bfloat16)
    W = torch.randn((N, K), generator=g).to(dev).to(torch.bfloat16)
    b = torch.randn(N, generator=g).to(dev)
    z = A.float() @ W.float().T + b
    out = {}
    for flags in (0, 2):
        if epi == "f32":
            Cf = torch.zeros((M, N), dtype=torch.float32, device=dev)
            SG.gemm(A, True, W, True, Cf, M, N, K, bias=b if splitk == 1 else None, splitk=splitk, flags=flags)
            out[flags] = (Cf,)
        elif epi == "gelu":
            H = torch.empty((M, N), dtype=torch.bfloat16, device=dev)
            Z = torch.empty_like(H)
            SG.gemm(A, True, W, True, H, M, N, K, bias=b, gelu=True, Z=Z, flags=flags)
            out[flags] = (H, Z)
        else:
            ss = torch.zeros(N, dtype=torch.float32, device=dev)
            C.check(C.load().oneka_gemm_bf16_sigmoid_colsum(C.ptr(A), K, C.ptr(W), K, C.ptr(b), C.ptr(ss), M, N, K,
                                                             flags, C.stream_ptr()))
            out[flags] = (ss,)
        torch.cuda.synchronize()
        assert SG.tc_status() == 0
    for x, y in zip(out[0], out[2]):
        if splitk > 1 or epi == "sigsum":     # atomic additions in another order
            assert torch.allclose(x, y, rtol=1e-5, atol=1e-4), float((x - y).abs().max())
        else:
            assert torch.equal(x, y), float((x.float() - y.float()).abs().max())
    if epi == "f32":
        ref = z if splitk == 1 else z - b
        assert torch.allclose(out[0][0], ref, rtol=1e-3, atol=2e-3), float((out[0][0] - ref).abs().max())
    elif epi == "gelu":
        assert torch.allclose(out[0][1].float(), z, rtol=2e-2, atol=2e-2)
        assert torch.allclose(out[0][0].float(), torch.nn.functional.gelu(z), rtol=2e-2, atol=2e-2)
    else:
        ref = torch.sigmoid(z).sum(0)
        assert torch.allclose(out[0][0], ref, rtol=1e-3, atol=1e-2), float((out[0][0] - ref).abs().max())


@pytest.mark.parametrize("rows,cols,lds,ldd", [(512, 65536, 65536, 512), (96, 200, 208, 104), (7, 13, 16, 8),
                                               (130, 64, 64, 136)])
def test_transpose_bf16(rows, cols, lds, ldd):
    """oneka_transpose_bf16 against torch's transpose, padded leading dimensions untouched."""
    dev = C.device()
    src = torch.randn((rows, lds), device=dev).to(torch.bfloat16)
    dst = torch.full((cols, ldd), 7.0, dtype=torch.bfloat16, device=dev)
    C.check(C.load().oneka_transpose_bf16(C.ptr(src), rows, cols, lds, C.ptr(dst), ldd, C.stream_ptr()))
    torch.cuda.synchronize()
    assert torch.equal(dst[:, :rows], src[:, :cols].T)
    assert bool((dst[:, rows:] == 7.0).all())


@pytest.mark.parametrize("flags", [0, 1])
@pytest.mark.parametrize("M,N,K", [(256, 128, 64), (200, 520, 512)])
def test_gemm_gelu_epilogue(flags, M, N, K):
    dev = C.device()
    g = torch.Generator(device="cpu").manual_seed(3 + K)
    A = torch.randn((M, K), generator=g).to(dev).to(torch.bfloat16)
    W = (torch.randn((N, K), generator=g) / math.sqrt(K)).to(dev).to(torch.bfloat16)
    b = torch.randn(N, generator=g).to(dev)
    H = torch.empty((M, N), dtype=torch.bfloat16, device=dev)
    Z = torch.empty_like(H)
    SG.gemm(A, True, W, True, H, M, N, K, bias=b, gelu=True, Z=Z, flags=flags)
    assert SG.gemm_path(True, True, K, c_f32=False, gelu=True, has_z=True, flags=flags) == int(flags == 0)
    assert SG.tc_status() == 0
    z = A.float() @ W.float().T + b
    assert torch.allclose(Z.float(), z, rtol=2e-2, atol=2e-2)
    assert torch.allclose(H.float(), torch.nn.functional.gelu(z), rtol=2e-2, atol=2e-2)


def test_mlp_gradients_match_cpu_oracle():
    import mlp_oracle
    dev = C.device()
    dims = [64, 96, 96, 64, 512]
    model = SG.MLP(dims, dev, seed=1)
    Bn = 64
    g = torch.Generator(device="cpu").manual_seed(9)
    X = (torch.randn((Bn, 64), generator=g) * 0.8).to(dev).to(torch.bfloat16)
    # labels: a 16 x 32 grid per sample in the chronicle's bitmask layout
    bits = (torch.rand((Bn, 16, 32), generator=g) < 0.3)
    words = (bits.to(torch.int64) << torch.arange(32)).sum(-1)            # [B][16] one word per row
    masks = torch.where(words >= 2**31, words - 2**32, words).to(torch.int32).reshape(Bn, 16).to(dev)
    model.forward(X)
    loss = model.loss_and_grad(masks, 16, 1, 32)
    model.backward()
    torch.cuda.synchronize()
    W = [L.wb.float().cpu().double().numpy() for L in model.layers]
    bvec = [L.b.cpu().double().numpy() for L in model.layers]
    lo, dW, db = mlp_oracle.forward_backward(X.float().cpu().double().numpy(), W, bvec,
                                             bits.reshape(Bn, 512).double().numpy())
    assert abs(float(loss.item()) - lo) < 1e-3 * max(1.0, abs(lo))
    for i, L in enumerate(model.layers):
        gw = L.gw.cpu().double().numpy()
        gb = L.gb.cpu().double().numpy()
        assert np.linalg.norm(gw - dW[i]) <= 0.03 * np.linalg.norm(dW[i]) + 1e-12, i
        assert np.linalg.norm(gb - db[i]) <= 0.03 * np.linalg.norm(db[i]) + 1e-12, i


def test_transposing_bce_and_adamw_match_plain_kernels():
    """oneka_bce_bitmask_t and oneka_adamw_scheduled_t: the plain kernels'
    results, plus exact transposed BF16 copies."""
    dev = C.device()
    g = torch.Generator(device="cpu").manual_seed(8)
    B, nr, nc = 128, 8, 128
    ncells, wpr = nr * nc, nc // 32
    slot = nr * wpr
    logits = (torch.randn((B, ncells), generator=g) * 3).to(dev)
    masks = torch.randint(-2**31, 2**31 - 1, (B, slot), dtype=torch.int64, generator=g).to(torch.int32).to(dev)
    Lb = C.load()
    d1 = torch.empty((B, ncells), dtype=torch.bfloat16, device=dev)
    d2 = torch.empty_like(d1)
    dt = torch.empty((ncells, B), dtype=torch.bfloat16, device=dev)
    l1 = torch.zeros(1, device=dev)
    l2 = torch.zeros(1, device=dev)
    C.check(Lb.oneka_bce_bitmask(C.ptr(logits), C.ptr(masks), slot, wpr, nc, B, ncells, 1.0 / (B * ncells), C.ptr(d1),
                                 C.ptr(l1), C.stream_ptr()))
    C.check(Lb.oneka_bce_bitmask_t(C.ptr(logits), C.ptr(masks), slot, wpr, nc, B, ncells, 1.0 / (B * ncells),
                                   C.ptr(d2), C.ptr(dt), B, C.ptr(l2), C.stream_ptr()))
    torch.cuda.synchronize()
    assert torch.equal(d1, d2) and torch.equal(dt, d2.T)
    assert abs(float(l1) - float(l2)) <= 1e-5 * abs(float(l1))
    rows, cols = 192, 256
    w0 = (torch.randn((rows, cols), generator=g) * 0.05).to(dev)
    m0 = (torch.randn((rows, cols), generator=g) * 0.01).to(dev)
    v0 = (torch.rand((rows, cols), generator=g) * 0.01).to(dev)
    gr = torch.randn((rows, cols), generator=g).to(dev)
    hyper = torch.tensor([1e-3, 1 - 0.9 ** 3, 1 - 0.999 ** 3], dtype=torch.float32, device=dev)
    out = {}
    for t in (False, True):
        w, m, v = w0.clone(), m0.clone(), v0.clone()
        wb = torch.empty((rows, cols), dtype=torch.bfloat16, device=dev)
        wbt = torch.empty((cols, rows), dtype=torch.bfloat16, device=dev)
        if t:
            C.check(Lb.oneka_adamw_scheduled_t(C.ptr(w), C.ptr(m), C.ptr(v), C.ptr(gr), C.ptr(wb), C.ptr(wbt), rows,
                                               rows, cols, C.ptr(hyper), 0.9, 0.999, 1e-8, 1e-4, C.stream_ptr()))
        else:
            C.check(Lb.oneka_adamw_scheduled(C.ptr(w), C.ptr(m), C.ptr(v), C.ptr(gr), C.ptr(wb), rows * cols,
                                             C.ptr(hyper), 0.9, 0.999, 1e-8, 1e-4, C.stream_ptr()))
        torch.cuda.synchronize()
        out[t] = (w, m, v, wb, wbt)
    for a, b in zip(out[False][:3], out[True][:3]):     # the same update; multiply-adds may contract differently
        assert torch.allclose(a, b, rtol=1e-5, atol=1e-7), float((a - b).abs().max())
    assert torch.equal(out[True][4], out[True][3].T)
    assert float((out[True][3].float() - out[False][3].float()).abs().max()) <= 2 ** -8 * 0.3


def test_graph_captured_training_matches_eager():
    """SG.train with the training step captured as a CUDA graph (and its
    schedule read from the device by oneka_adamw_scheduled) follows the
    eager loop: same losses and weights up to the order of the split-K
    atomic sums."""
    dev = C.device()
    g = torch.Generator(device="cpu").manual_seed(5)
    X = (torch.randn((2048, 64), generator=g) * 0.8).to(dev).to(torch.bfloat16)
    bits = torch.rand((2048, 64, 64), generator=g) < 0.2
    words = (bits.reshape(2048, 64, 2, 32).to(torch.int64) << torch.arange(32)).sum(-1)
    masks = torch.where(words >= 2**31, words - 2**32, words).to(torch.int32).reshape(2048, 128).to(dev)
    runs = {}
    for graph in (False, True):
        model = SG.MLP([64, 256, 256, 4096], dev, seed=2, out_bias=-1.0)
        losses = SG.train(model, X, masks, 128, 2, 64, epochs=2, batch=256, lr=2e-3, lr_final=5e-4, graph=graph)
        torch.cuda.synchronize()
        runs[graph] = (losses, [L.w.clone() for L in model.layers])
    (l0, w0), (l1, w1) = runs[False], runs[True]
    assert len(l0) == len(l1) and l0[-1] < l0[0]
    assert np.allclose(l0, l1, rtol=1e-3, atol=1e-6), (l0, l1)
    for a, b in zip(w0, w1):
        assert float((a - b).norm() / a.norm()) < 1e-3


def test_adamw_matches_restatement():
    import mlp_oracle
    dev = C.device()
    g = torch.Generator(device="cpu").manual_seed(4)
    w = torch.randn(1000, generator=g)
    m = torch.randn(1000, generator=g) * 0.1
    v = torch.rand(1000, generator=g) * 0.1
    grad = torch.randn(1000, generator=g)
    wd, md, vd, gd = (t.to(dev).contiguous() for t in (w, m, v, grad))
    wb = torch.empty(1000, dtype=torch.bfloat16, device=dev)
    C.check(C.load().oneka_adamw(C.ptr(wd), C.ptr(md), C.ptr(vd), C.ptr(gd), C.ptr(wb), 1000, 1e-3, 0.9, 0.999,
                                 1e-8, 1e-2, 7, C.stream_ptr()))
    w2, m2, v2 = mlp_oracle.adamw(w.double().numpy(), m.double().numpy(), v.double().numpy(),
                                  grad.double().numpy(), 1e-3, 0.9, 0.999, 1e-8, 1e-2, 7)
    assert np.allclose(wd.cpu().numpy(), w2, rtol=1e-5, atol=1e-6)
    assert np.allclose(md.cpu().numpy(), m2, rtol=1e-5, atol=1e-6)
    assert torch.equal(wb, wd.to(torch.bfloat16))


@pytest.mark.parametrize("flags", [0, 1])
def test_fused_sigmoid_colsum_matches_fp32(flags):
    dev = C.device()
    g = torch.Generator(device="cpu").manual_seed(11)
    for M, N, K in [(300, 520, 64), (2048, 4096, 256), (130, 65536, 512)]:
        H = torch.randn((M, K), generator=g).to(dev).to(torch.bfloat16)
        W = (torch.randn((N, K), generator=g) * 0.2).to(dev).to(torch.bfloat16)
        b = torch.randn(N, generator=g).to(dev)
        out = torch.full((N,), 0.5, dtype=torch.float32, device=dev)
        C.check(C.load().oneka_gemm_bf16_sigmoid_colsum(C.ptr(H), K, C.ptr(W), K, C.ptr(b), C.ptr(out), M, N, K,
                                                        flags, C.stream_ptr()))
        assert SG.tc_status() == 0
        ref = 0.5 + torch.sigmoid(H.float() @ W.float().T + b).sum(0)
        assert torch.allclose(out, ref, rtol=1e-4, atol=1e-3 * math.sqrt(M)), float((out - ref).abs().max())


def test_trained_surrogate_screens_faster_within_tolerance():
    """Train on tracker-chronicled masks of the 31-well site (1000 paths, 20
    years, a 128 x 128 grid at 20 m, 64 k realizations), then screen 16 k
    fresh realizations with 25 % judges: the judges accept the surrogate at
    the tracker's own bar (L-inf <= 0.01), the screened field agrees with
    tracking every realization, and screening costs less than tracking
    everything.  (The judges' L-inf includes their sampling noise, about
    sqrt(p (1 - p) / n) per cell, hence 4,096 judges.)"""
    dev = C.device()
    spec = S.config5(npaths=1000)
    site = E.Site(spec.wells, spec.observations, spec.base, c_dist=spec.c_dist, p_dist=spec.p_dist,
                  t_dist=spec.t_dist, device=dev)
    nr = nc = 128
    grid = E.Grid(site.xt - 1270.0, site.yt - 1270.0, 20.0, 20.0, nr, nc)
    release = torch.as_tensor(site.release(spec.npaths), device=dev)
    opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=False, precision=C.FP32)
    train_real = E.realize(site, 65536, seed=77)
    masks, slot_words = SG.chronicle_masks(site, train_real, release, opts, grid)
    feats = SG.Features(train_real, site.nwells)
    X = feats(train_real)
    model = SG.MLP([64, 512, 512, 512, nr * nc], dev, seed=3, out_bias=math.log(0.05 / 0.95))
    losses = SG.train(model, X, masks, slot_words, grid.words_per_row, nc, epochs=8, batch=512, lr=1.5e-3,
                      lr_final=1e-4)
    assert losses[-1] < 0.5 * losses[0], losses
    fresh = E.realize(site, 16384, seed=78)
    SG.screen(model, feats, site, fresh.slice(0, 1024), release, opts, grid, judge_fraction=0.25,
              tolerance=1.0)                                   # warm-up
    # the acceptance bar is the FP32 tracker's own: L-inf <= 0.01 over the judges
    res = SG.screen(model, feats, site, fresh, release, opts, grid, judge_fraction=0.25, tolerance=0.01)
    assert res.accepted, (res.judge_linf, res.judge_l1)
    counts = torch.zeros((nr, nc), dtype=torch.int32, device=dev)
    E.track(site, fresh.slice(0, 1024), release, opts, grid, counts=counts)   # warm-up
    counts.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    E.track(site, fresh, release, opts, grid, counts=counts)
    e1.record()
    torch.cuda.synchronize()
    t_track = e0.elapsed_time(e1) / 1e3
    full = counts.double() / fresh.n
    err = (res.field - full).abs()
    print(f"surrogate screen: loss {losses[0]:.4f} -> {losses[-1]:.4f}; judges {res.n_judges} "
          f"L-inf {res.judge_linf:.4f} L1 {res.judge_l1:.2e}; field vs all-tracked L-inf "
          f"{float(err.max()):.4f} L1 {float(err.mean()):.2e}; screen {res.seconds * 1e3:.1f} ms "
          f"(judges {res.seconds_judges * 1e3:.1f}, surrogate {res.seconds_surrogate * 1e3:.1f}) vs "
          f"track-all {t_track * 1e3:.1f} ms")
    assert float(err.max()) < 0.02
    assert res.seconds < t_track, (res.seconds, t_track)


def test_untrained_surrogate_is_rejected_and_every_realization_tracked():
    """An untrained network fails the judges (L-inf above the tolerance);
    screen() then tracks every realization, and the field equals tracking
    them all directly, node for node."""
    dev = C.device()
    spec = S.config5(npaths=200)
    site = E.Site(spec.wells, spec.observations, spec.base, c_dist=spec.c_dist, p_dist=spec.p_dist,
                  t_dist=spec.t_dist, device=dev)
    grid = E.Grid(site.xt - 630.0, site.yt - 630.0, 20.0, 20.0, 64, 64)
    release = torch.as_tensor(site.release(spec.npaths), device=dev)
    opts = E.TrackOptions(duration=5 * 365.25, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=False, precision=C.FP32)
    real = E.realize(site, 600, seed=21)
    feats = SG.Features(real, site.nwells)
    model = SG.MLP([64, 64, 64, 64 * 64], dev, seed=1, out_bias=2.0)      # sigmoid(2) = 0.88 everywhere
    res = SG.screen(model, feats, site, real, release, opts, grid, judge_fraction=0.05, tolerance=0.01)
    assert not res.accepted and res.judge_linf > 0.01
    counts = torch.zeros((64, 64), dtype=torch.int32, device=dev)
    E.track(site, real, release, opts, grid, counts=counts)
    assert torch.equal(res.field, counts.double().reshape(64, 64) / real.n)
