"""Learned surrogate of the tracker: realization parameters -> capture logits.

An MLP (features 39 -> 512 -> 512 -> 512 GELU -> 256 x 256 logits) maps a
realization's parameter vector (A..F, the discharges, K, porosity) to
per-cell capture logits on the site grid.  It is trained in BF16 with FP32
master weights on (parameters -> visited-cell mask) pairs that the tracker
itself chronicles (oneka_track mark-only mode: one bitmask per realization),
with the project's own kernels: oneka_gemm_bf16 (tensor cores),
oneka_bce_bitmask(_t), oneka_transpose_bf16, oneka_gelu_backward,
oneka_colsum_bf16, oneka_adamw_scheduled(_t).

Screening: the surrogate's field is the mean of sigmoid(logits) over the
screened realizations; a held-out fraction (the judges) is always tracked,
and the surrogate's field over the judges is compared with their tracked
field.  The surrogate is rejected -- the run falls back to tracking every
realization -- when that L-inf error exceeds the stated tolerance.

No counterpart in the reference.
"""
from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass

import torch

from . import _capi as C
from . import engine as E

BF16 = torch.bfloat16
F32 = torch.float32


def _p(t):
    return C.ptr(t)


# flags of oneka_gemm_bf16: bit 0 forces the mma.sync kernel (default: the
# tcgen05 kernel wherever it applies).
GEMM_FLAGS = 0
SM_COUNT = 152          # split-K targets about two work items per SM of a GB300


def gemm(A, a_kmajor, B, b_kmajor, C_out, M, N, K, *, bias=None, gelu=False, Z=None, splitk=1, stream=None,
         flags=None):
    lda = A.shape[-1]
    ldb = B.shape[-1]
    ldc = C_out.shape[-1]
    C.check(C.load().oneka_gemm_bf16(_p(A), lda, int(a_kmajor), _p(B), ldb, int(b_kmajor), _p(C_out), ldc,
                                     int(C_out.dtype == F32), _p(bias), int(gelu), _p(Z), M, N, K, splitk,
                                     GEMM_FLAGS if flags is None else flags, C.stream_ptr(stream)))


def gemm_path(a_kmajor, b_kmajor, K, *, splitk=1, c_f32=True, gelu=False, has_z=False, sigsum=False, flags=None):
    """1 when the GEMM runs on the tcgen05 kernel, 0 on the mma.sync kernel."""
    return int(C.load().oneka_gemm_bf16_path(int(a_kmajor), int(b_kmajor), K, splitk, int(c_f32), int(gelu),
                                             int(has_z), int(sigsum), GEMM_FLAGS if flags is None else flags))


def tc_status() -> int:
    """Device status of the tcgen05 GEMM (0 ok, 1 a wait timed out); clears it."""
    v = ctypes.c_int32(0)
    C.check(C.load().oneka_gemm_tc_status(ctypes.byref(v)))
    return int(v.value)


@dataclass
class Layer:
    w: torch.Tensor        # FP32 master [out][in]
    b: torch.Tensor        # FP32 [out]
    wb: torch.Tensor       # BF16 copy [out][in]
    mw: torch.Tensor
    vw: torch.Tensor
    mb: torch.Tensor
    vb: torch.Tensor
    gw: torch.Tensor       # FP32 gradients
    gb: torch.Tensor
    wbt: torch.Tensor | None = None   # BF16 W^T [in][out] for the backward pass
    wbt_valid: bool = False            # wbt equals wb^T (kept by oneka_adamw_scheduled_t)


class MLP:
    """dims = [in, h, h, h, out]; hidden layers use GELU."""

    def __init__(self, dims, device, seed=0, out_bias=0.0):
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.dims = list(dims)
        self.layers = []
        for i, (din, dout) in enumerate(zip(dims[:-1], dims[1:])):
            std = math.sqrt(2.0 / din) if i < len(dims) - 2 else math.sqrt(1.0 / din) * 0.5
            w = (torch.randn((dout, din), generator=g) * std).to(device)
            b = torch.full((dout,), out_bias if i == len(dims) - 2 else 0.0).to(device)
            self.layers.append(Layer(w, b, w.to(BF16), torch.zeros_like(w), torch.zeros_like(w),
                                     torch.zeros_like(b), torch.zeros_like(b), torch.zeros_like(w),
                                     torch.zeros_like(b)))
        self.step_count = 0
        self._acts = {}

    def _buffers(self, B, device):
        key = B
        if key not in self._acts:
            self._acts[key] = dict(
                H=[torch.empty((B, d), dtype=BF16, device=device) for d in self.dims[1:-1]],
                Z=[torch.empty((B, d), dtype=BF16, device=device) for d in self.dims[1:-1]],
                logits=torch.empty((B, self.dims[-1]), dtype=F32, device=device),
                dlogits=torch.empty((B, self.dims[-1]), dtype=BF16, device=device),
                dh=[torch.empty((B, d), dtype=F32, device=device) for d in self.dims[1:-1]],
                dz=[torch.empty((B, d), dtype=BF16, device=device) for d in self.dims[1:-1]])
        return self._acts[key]

    def _hidden(self, X):
        """GELU layers; returns the last hidden activations (BF16)."""
        a = self._buffers(X.shape[0], X.device)
        h = X
        for i, L in enumerate(self.layers[:-1]):
            dout, din = L.w.shape
            gemm(h, True, L.wb, True, a["H"][i], X.shape[0], dout, din, bias=L.b, gelu=True, Z=a["Z"][i])
            h = a["H"][i]
        return h

    def forward(self, X):
        """X: BF16 [B][in].  Returns FP32 logits [B][out] (kept for backward)."""
        a = self._buffers(X.shape[0], X.device)
        h = self._hidden(X)
        L = self.layers[-1]
        gemm(h, True, L.wb, True, a["logits"], X.shape[0], L.w.shape[0], L.w.shape[1], bias=L.b)
        self._X = X
        return a["logits"]

    def loss_and_grad(self, masks, slot_words, wpr, ncols):
        """BCE against chronicle bitmasks (rows of slot_words words) and dlogits."""
        a = self._buffers(self._X.shape[0], self._X.device)
        B, ncells = a["logits"].shape
        if "loss" not in a:
            a["loss"] = torch.zeros(1, dtype=F32, device=self._X.device)
        loss = a["loss"]
        loss.zero_()
        if B % 64 == 0 and ncols % 64 == 0:
            # the gradient also transposed, [ncells][B]: the last layer's weight-gradient operand
            if "dlogits_t" not in a:
                a["dlogits_t"] = torch.empty((ncells, B), dtype=BF16, device=self._X.device)
            C.check(C.load().oneka_bce_bitmask_t(_p(a["logits"]), _p(masks), slot_words, wpr, ncols, B, ncells,
                                                 1.0 / (B * ncells), _p(a["dlogits"]), _p(a["dlogits_t"]), B,
                                                 _p(loss), C.stream_ptr()))
            self._dlogits_t = True
        else:
            C.check(C.load().oneka_bce_bitmask(_p(a["logits"]), _p(masks), slot_words, wpr, ncols, B, ncells,
                                               1.0 / (B * ncells), _p(a["dlogits"]), _p(loss), C.stream_ptr()))
            self._dlogits_t = False
        return loss

    def _transposed(self, name, rows, cols, device):
        key = ("T", name, rows, cols)
        if key not in self._acts:
            self._acts[key] = torch.empty((cols, rows), dtype=BF16, device=device)
        return self._acts[key]

    def backward(self, hyper=None, betas=(0.9, 0.999), eps=1e-8, weight_decay=1e-4):
        """Gradients of every layer, and with `hyper` (device [lr, 1 - beta1^t,
        1 - beta2^t]) the AdamW step too.

        The two GEMMs per layer contract over the batch (gW = dZ^T H_in) and
        over the layer's outputs (dH_in = dZ W); their operands are stored with
        the contracted index outermost, so they run K-major on the tensor
        cores from transposed copies: dZ^T of the last layer comes from the
        loss kernel, W^T from the previous AdamW step (oneka_adamw_scheduled_t
        keeps it), the rest from oneka_transpose_bf16.  A GEMM with fewer
        output tiles than SMs is split over K.  A layer's dH_in is computed
        before its weights are stepped."""
        X = self._X
        B = X.shape[0]
        dev = X.device
        a = self._buffers(B, dev)
        n = len(self.layers)
        Lb = C.load()
        dcur = a["dlogits"]                    # BF16 dZ of the current layer
        for i in range(n - 1, -1, -1):
            L = self.layers[i]
            dout, din = L.w.shape
            hin = X if i == 0 else a["H"][i - 1]
            # gW = dZ^T H_in : [dout][din] = (dZ^T [dout][B]) (H_in^T [din][B])^T
            if i == n - 1 and getattr(self, "_dlogits_t", False):
                dzt = a["dlogits_t"]
            else:
                dzt = self._transposed(("dz", i), B, dout, dev)
                C.check(Lb.oneka_transpose_bf16(_p(dcur), B, dout, dcur.shape[-1], _p(dzt), B, C.stream_ptr()))
            hint = self._transposed(("h", i), B, din, dev)
            C.check(Lb.oneka_transpose_bf16(_p(hin), B, din, hin.shape[-1], _p(hint), B, C.stream_ptr()))
            tiles_w = -(-dout // 128) * -(-din // 256)
            splitk = max(1, min(B // 64, round(2 * SM_COUNT / tiles_w))) if B % 64 == 0 else 1
            if splitk > 1:
                L.gw.zero_()
            gemm(dzt, True, hint, True, L.gw, dout, din, B, splitk=splitk)
            C.check(Lb.oneka_colsum_bf16(_p(dcur), B, dout, _p(L.gb), C.stream_ptr()))
            dz = None
            if i > 0:
                # dH_in = dZ W : [B][din] = (dZ [B][dout]) (W^T [din][dout])^T, split over K = dout
                wt = self._weight_t(L)
                dh = a["dh"][i - 1]
                dh.zero_()
                tiles = -(-B // 128) * -(-din // 256)
                splitk = max(1, min(dout // 64, round(2 * SM_COUNT / tiles)))
                gemm(dcur, True, wt, True, dh, B, din, dout, splitk=splitk)
                dz = a["dz"][i - 1]
                C.check(Lb.oneka_gelu_backward(_p(dh), _p(a["Z"][i - 1]), _p(dz), dh.numel(), C.stream_ptr()))
            if hyper is not None:
                self._step_layer(L, hyper, betas, eps, weight_decay)
            if dz is None:
                break
            dcur = dz

    def _step_layer(self, L, hyper, betas, eps, weight_decay):
        """AdamW step of one layer's weights and bias (schedule in `hyper`)."""
        Lb = C.load()
        dout, din = L.w.shape
        if dout % 64 == 0 and din % 64 == 0:       # the step keeps W^T current
            C.check(Lb.oneka_adamw_scheduled_t(_p(L.w), _p(L.mw), _p(L.vw), _p(L.gw), _p(L.wb), _p(self._wt_buffer(L)),
                                               dout, dout, din, _p(hyper), betas[0], betas[1], eps, weight_decay,
                                               C.stream_ptr()))
            L.wbt_valid = True
        else:
            C.check(Lb.oneka_adamw_scheduled(_p(L.w), _p(L.mw), _p(L.vw), _p(L.gw), _p(L.wb), L.w.numel(), _p(hyper),
                                             betas[0], betas[1], eps, weight_decay, C.stream_ptr()))
            L.wbt_valid = False
        C.check(Lb.oneka_adamw_scheduled(_p(L.b), _p(L.mb), _p(L.vb), _p(L.gb), None, L.b.numel(), _p(hyper),
                                         betas[0], betas[1], eps, 0.0, C.stream_ptr()))

    def _wt_buffer(self, L):
        if getattr(L, "wbt", None) is None:
            L.wbt = torch.empty((L.w.shape[1], L.w.shape[0]), dtype=BF16, device=L.w.device)
            L.wbt_valid = False
        return L.wbt

    def _weight_t(self, L):
        """W^T of layer L in BF16 [din][dout], transposed now unless an
        oneka_adamw_scheduled_t step has kept it current."""
        wt = self._wt_buffer(L)
        if not getattr(L, "wbt_valid", False):
            dout, din = L.w.shape
            C.check(C.load().oneka_transpose_bf16(_p(L.wb), dout, din, din, _p(wt), dout, C.stream_ptr()))
        return wt

    def adamw(self, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=1e-4):
        self.step_count += 1
        Lb = C.load()
        for L in self.layers:
            L.wbt_valid = False
            C.check(Lb.oneka_adamw(_p(L.w), _p(L.mw), _p(L.vw), _p(L.gw), _p(L.wb), L.w.numel(), lr, betas[0],
                                   betas[1], eps, weight_decay, self.step_count, C.stream_ptr()))
            C.check(Lb.oneka_adamw(_p(L.b), _p(L.mb), _p(L.vb), _p(L.gb), None, L.b.numel(), lr, betas[0],
                                   betas[1], eps, 0.0, self.step_count, C.stream_ptr()))

    def adamw_scheduled(self, hyper, betas=(0.9, 0.999), eps=1e-8, weight_decay=1e-4):
        """AdamW with the step's lr and bias corrections read from the device
        tensor hyper = [lr, 1 - beta1^t, 1 - beta2^t] (a captured step)."""
        Lb = C.load()
        for L in self.layers:
            L.wbt_valid = False
            C.check(Lb.oneka_adamw_scheduled(_p(L.w), _p(L.mw), _p(L.vw), _p(L.gw), _p(L.wb), L.w.numel(),
                                             _p(hyper), betas[0], betas[1], eps, weight_decay, C.stream_ptr()))
            C.check(Lb.oneka_adamw_scheduled(_p(L.b), _p(L.mb), _p(L.vb), _p(L.gb), None, L.b.numel(), _p(hyper),
                                             betas[0], betas[1], eps, 0.0, C.stream_ptr()))

    def sigmoid_sum(self, X, out):
        """out[c] += sum over rows of sigmoid(logits) (the screened visits);
        the last layer's GEMM sums in its epilogue, logits are not stored."""
        h = self._hidden(X)
        L = self.layers[-1]
        C.check(C.load().oneka_gemm_bf16_sigmoid_colsum(_p(h), h.shape[-1], _p(L.wb), L.wb.shape[-1], _p(L.b),
                                                        _p(out), X.shape[0], L.w.shape[0], L.w.shape[1],
                                                        GEMM_FLAGS, C.stream_ptr()))


# ---------------------------------------------------------------------------
class Features:
    """Feature standardization (A..F, discharges, K, porosity) into BF16 rows of `ld`."""

    def __init__(self, real: E.Realizations, nwells: int, ld: int = 64):
        raw = torch.cat([real.coef, real.q, real.aquifer[:, :2]], dim=1).float()
        self.nf = raw.shape[1]
        self.mean = raw.mean(dim=0).contiguous()
        sd = raw.std(dim=0)
        self.inv_std = torch.where(sd > 0, 1.0 / sd, torch.ones_like(sd)).contiguous()
        self.nwells = nwells
        self.ld = ld

    def __call__(self, real: E.Realizations, out=None):
        n = real.n
        if out is None:
            out = torch.empty((n, self.ld), dtype=BF16, device=real.coef.device)
        C.check(C.load().oneka_features(_p(real.coef), _p(real.q), _p(real.aquifer), self.nwells, n,
                                        _p(self.mean), _p(self.inv_std), self.nf, self.ld, _p(out),
                                        C.stream_ptr()))
        return out


def chronicle_masks(site: E.Site, real: E.Realizations, release, opts: E.TrackOptions, grid: E.Grid):
    """One chronicle bitmask per realization (the training labels): the
    tracker in mark-only mode.  Returns (masks int32 [n][slot_words], slot_words)."""
    slot_words = grid.slot_bytes() // 4
    masks = torch.zeros((real.n, slot_words), dtype=torch.int32, device=site.device)
    E.track(site, real, release, opts, grid, mark_only=masks)
    return masks, slot_words


@dataclass
class ScreenResult:
    field: torch.Tensor            # screened capture probability [nrows][ncols]
    judge_linf: float              # L-inf of the surrogate vs tracked field over the judges
    judge_l1: float                # mean absolute difference over the judges
    accepted: bool                 # judge_linf <= tolerance
    n_screened: int
    n_judges: int
    seconds: float                 # wall time of the whole screen
    seconds_judges: float          # tracking the judges
    seconds_surrogate: float       # the surrogate over judges and screened realizations


def screen(model: MLP, feats: Features, site: E.Site, real: E.Realizations, release, opts: E.TrackOptions,
           grid: E.Grid, *, judge_fraction=0.05, tolerance=0.05, batch=2048, seed=0) -> ScreenResult:
    """Capture probability of `real` with the surrogate, a held-out `judge_fraction`
    always tracked.  If the judges disagree by more than `tolerance` (L-inf),
    every realization is tracked instead."""
    dev = site.device
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n = real.n
    nj = max(1, int(round(judge_fraction * n)))
    ncells = grid.nrows * grid.ncols
    # judges: the first nj realizations (every realization is an independent draw)
    judges = real.slice(0, nj)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    E.track(site, judges, release, opts, grid, counts=counts)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    surr = torch.zeros((2, ncells), dtype=F32, device=dev)   # [judges, the rest]
    for a in range(0, nj, batch):
        model.sigmoid_sum(feats(real.slice(a, min(nj, a + batch))), surr[0])
    for a in range(nj, n, batch):
        model.sigmoid_sum(feats(real.slice(a, min(n, a + batch))), surr[1])
    tracked_j = counts.reshape(-1).float() / nj
    diff = (surr[0] / nj - tracked_j).abs()
    stats = torch.stack([diff.max(), diff.mean()]).cpu()
    t2 = time.perf_counter()
    linf, l1 = float(stats[0]), float(stats[1])
    accepted = linf <= tolerance
    total = counts.reshape(-1).double()
    if accepted:
        total += surr[1].double()
    else:
        rest_counts = torch.zeros_like(counts)
        E.track(site, real.slice(nj, n), release, opts, grid, counts=rest_counts)
        total += rest_counts.reshape(-1).double()
    field = (total / n).reshape(grid.nrows, grid.ncols)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    return ScreenResult(field, linf, l1, accepted, n - nj, nj, t3 - t0, t1 - t0, t2 - t1)


def train(model: MLP, X: torch.Tensor, masks: torch.Tensor, slot_words: int, wpr: int, ncols: int, *,
          epochs=3, batch=512, lr=1e-3, weight_decay=1e-4, lr_final=1e-4, log=None, graph=True):
    """Mini-batch AdamW over consecutive batches (realizations are i.i.d. draws).

    With `graph` the training step (forward, loss, backward, AdamW: about 40
    kernel launches) is captured once as a CUDA graph after one eager step
    and replayed for every later batch; each batch is first copied into the
    graph's fixed input buffers, and the step's learning rate and bias
    corrections into a device tensor that the AdamW kernels read."""
    n = X.shape[0]
    nb = n // batch
    total = epochs * nb
    betas, eps = (0.9, 0.999), 1e-8
    dev = X.device
    xs = torch.empty((batch, X.shape[1]), dtype=X.dtype, device=dev)
    ms = torch.empty((batch, masks.shape[1]), dtype=masks.dtype, device=dev)
    hyper = torch.zeros(3, dtype=F32, device=dev)

    def body():
        model.forward(xs)
        model.loss_and_grad(ms, slot_words, wpr, ncols)
        model.backward(hyper, betas, eps, weight_decay)     # gradients and the AdamW step

    g = None
    losses = []
    for ep in range(epochs):
        for k in range(nb):
            step = ep * nb + k
            frac = step / max(1, total - 1)
            lr_k = lr * (lr_final / lr) ** frac          # exponential decay to lr_final
            model.step_count += 1
            t = model.step_count
            xs.copy_(X[k * batch:(k + 1) * batch], non_blocking=True)
            ms.copy_(masks[k * batch:(k + 1) * batch], non_blocking=True)
            hyper.copy_(torch.tensor([lr_k, 1.0 - betas[0] ** t, 1.0 - betas[1] ** t], dtype=F32).pin_memory(),
                        non_blocking=True)
            if not graph:
                body()
            elif g is None:
                body()                                   # one eager step: buffers, kernels and maps set up
                torch.cuda.synchronize()
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    body()
            else:
                g.replay()
            if k % 50 == 0 or k == nb - 1:
                losses.append(float(model._buffers(batch, dev)["loss"].item()))
                if log:
                    log(ep, k, losses[-1])
    return losses
