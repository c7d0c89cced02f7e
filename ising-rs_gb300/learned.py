"""Learned autoregressive proposal: training on sampler configurations and an
exact Metropolis-Hastings chain that interleaves checkerboard sweeps.

No reference counterpart (faulknco/ising-rs has no learned sampler).  The
network and its kernels live in csrc/isg_learned.cu; this module drives them
through the C ABI.  Device buffers are torch tensors on the library's stream.

The chain at temperature T on a periodic L^dim lattice alternates:
  * `sweeps` checkerboard sweeps of the current state (the Ising engine), and
  * one batch of K proposals y ~ q_sym, each tested in order by the
    independence Metropolis-Hastings rule (accept iff log u < A(y) - A(x),
    A = -beta E - log q_sym).
Both moves leave exp(-beta E) invariant.  The plain sampler is the fallback:
during the first `burn_in` batches, a batch whose acceptance falls below
`min_accept` is followed by `fallback_sweeps` sweeps instead of `sweeps`.
After burn-in the number of sweeps per batch is frozen (`fallback_sweeps` if
the mean burn-in acceptance is below `min_accept`, else `sweeps`): a rule that
kept reading the chain's own acceptance would choose the next kernel from the
current state, and the composite chain would no longer leave exp(-beta E)
invariant.  Samples taken after burn-in are exact.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import IsingBatch, IsingError, _check, _ptr, lib  # noqa: F401  (package-relative)


def _declare_learned(L):
    vp, i32, i64, u64, dbl, f32 = C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double, C.c_float
    sig = {
        "isg_learned_create": [C.POINTER(vp), i32, i32, i32, u64],
        "isg_learned_create2": [C.POINTER(vp), i32, i32, i32, i32, u64],
        "isg_learned_destroy": [vp],
        "isg_learned_num_params": [vp, vp],
        "isg_learned_get_weights": [vp, vp],
        "isg_learned_set_weights": [vp, vp],
        "isg_learned_gradient": [vp, vp, i32, vp, vp],
        "isg_learned_train": [vp, vp, i32, i32, i32, f32, vp],
        "isg_learned_sample": [vp, i32, u64, vp, vp, vp],
        "isg_learned_score": [vp, vp, i32, i32, vp],
        "isg_learned_batch_quantum": [vp, vp],
        "isg_learned_energies": [vp, vp, i32, i32, i32, vp, vp],
        "isg_learned_imh": [vp, vp, vp, vp, vp, i32, dbl, dbl, vp, vp, vp, vp, vp, vp, u64],
        "isg_learned_state_a": [vp, vp, vp, vp, dbl, dbl, vp],
        "isg_learned_adopt": [vp, vp, vp, vp],
        "isg_learned_sync": [vp],
        "isg_ising_load_natural": [vp, i32, i32, vp],
        "isg_ising_store_natural": [vp, i32, i32, vp],
        "isg_ising_store_natural_all": [vp, i32, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = i32
    L.isg_learned_stream.argtypes = [vp]
    L.isg_learned_stream.restype = vp


def _lib():
    L = lib()
    if not getattr(L, "_learned_declared", False):
        _declare_learned(L)
        L._learned_declared = True
    return L


def _tptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class LearnedProposal:
    """Masked-conv autoregressive network over an H x W raster of +-1 spins;
    zrow > 0 (a 3D lattice's L^2 x L raster: zrow = L) adds layer 0's z-plane
    tap (isg_learned_create2)."""

    def __init__(self, H: int, W: int, layers: int = 6, seed: int = 7, zrow: int = 0):
        self.H, self.W, self.layers, self.seed = int(H), int(W), int(layers), int(seed)
        self.zrow = int(zrow)
        h = C.c_void_p()
        _check(_lib().isg_learned_create2(C.byref(h), self.H, self.W, self.zrow, self.layers,
                                          self.seed))
        self._h = h
        n = C.c_int()
        _check(_lib().isg_learned_num_params(self._h, C.byref(n)))
        self.n_params = n.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib().isg_learned_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream_handle(self) -> int:
        return int(_lib().isg_learned_stream(self._h) or 0)

    def torch_stream(self):
        import torch
        return torch.cuda.ExternalStream(self.stream_handle)

    def weights(self) -> np.ndarray:
        w = np.zeros(self.n_params, np.float32)
        _check(_lib().isg_learned_get_weights(self._h, _ptr(w)))
        return w

    def set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, np.float32)
        _check(_lib().isg_learned_set_weights(self._h, _ptr(w)))

    def gradient(self, cfg) -> tuple[np.ndarray, float]:
        """Mean NLL of host configurations (B, H*W) int8 and its gradient."""
        cfg = np.ascontiguousarray(cfg, np.int8).reshape(-1, self.H * self.W)
        g = np.zeros(self.n_params, np.float32)
        nll = C.c_float()
        _check(_lib().isg_learned_gradient(self._h, _ptr(cfg), cfg.shape[0], _ptr(g),
                                           C.byref(nll)))
        return g, nll.value

    def train(self, d_cfg, batch: int = 256, steps: int = 100, lr: float = 1e-3) -> float:
        """Adam on device configurations d_cfg (torch int8, shape (n, H*W)); returns
        the mean log q of the last batch."""
        v = C.c_float()
        _check(_lib().isg_learned_train(self._h, _tptr(d_cfg), int(d_cfg.shape[0]), int(batch),
                                        int(steps), float(lr), C.byref(v)))
        return v.value

    def sample(self, K: int, step: int):
        """K samples (torch int8 (K, H*W)), log q, log q of the negations."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        out = torch.empty((K, self.H * self.W), dtype=torch.int8, device=dev)
        lq = torch.empty(K, dtype=torch.float32, device=dev)
        lqf = torch.empty(K, dtype=torch.float32, device=dev)
        _check(_lib().isg_learned_sample(self._h, int(K), int(step), _tptr(out), _tptr(lq),
                                         _tptr(lqf)))
        return out, lq, lqf

    def batch_quantum(self) -> int:
        """Proposals per full wave of the sampling kernel on this GPU."""
        v = C.c_int(0)
        _check(_lib().isg_learned_batch_quantum(self._h, C.byref(v)))
        return v.value

    def score(self, d_cfg, flip: bool = False):
        import torch
        lq = torch.empty(d_cfg.shape[0], dtype=torch.float32, device=d_cfg.device)
        _check(_lib().isg_learned_score(self._h, _tptr(d_cfg), int(d_cfg.shape[0]),
                                        1 if flip else 0, _tptr(lq)))
        return lq

    def sync(self):
        _check(_lib().isg_learned_sync(self._h))


class LearnedChain:
    """Exact MCMC at temperature T: learned independence proposals + sweeps."""

    def __init__(self, proposal: LearnedProposal, L: int, dim: int, T: float, J: float = 1.0,
                 K: int | None = 4096, sweeps: int = 1, fallback_sweeps: int = 20,
                 min_accept: float = 0.002, seed: int = 11, burn_in: int = 4):
        import torch
        self.q, self.L, self.dim, self.T, self.J = proposal, int(L), int(dim), float(T), float(J)
        if K is None:
            # at least 4096 proposals, in whole waves of the sampling kernel
            qn = proposal.batch_quantum()
            K = -(-4096 // qn) * qn
        self.K, self.sweeps, self.fallback, self.min_accept = int(K), int(sweeps), \
            int(fallback_sweeps), float(min_accept)
        self.burn_in = int(burn_in)
        self.n = self.L ** self.dim
        if self.n != proposal.H * proposal.W:
            raise IsingError(-1, "lattice size does not match the proposal raster")
        self.beta = 1.0 / self.T
        dev = torch.device("cuda", torch.cuda.current_device())
        self.dev = dev
        self.ising = IsingBatch([self.L], 1, seed=seed, dim=self.dim)
        self.ising.set_stream(proposal.stream_handle)
        self.ising.set_temperatures([self.T], J=self.J)
        self.cur = torch.empty(self.n, dtype=torch.int8, device=dev)
        self.state = torch.zeros(3, dtype=torch.int64, device=dev)
        self.ax = torch.zeros(1, dtype=torch.float64, device=dev)
        self.accepted = torch.zeros(1, dtype=torch.int64, device=dev)
        self.work = torch.empty(2 * self.K, dtype=torch.float64, device=dev)
        self.bond = torch.empty(self.K, dtype=torch.int64, device=dev)
        self.mag = torch.empty(self.K, dtype=torch.int64, device=dev)
        self.step_no = 0
        self._acc_prev = 0
        self.next_sweeps = self.sweeps
        self.records = []
        self.brecords = []
        self.batch_accept = []
        self.proposals = 0

    def close(self):
        """Give the Ising batch back its own stream and release it while the
        proposal (owner of the borrowed stream) is still alive."""
        b = getattr(self, "ising", None)
        if b is not None and getattr(b, "_h", None) and b._h.value:
            b.set_stream(None)
            b.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _refresh_state(self):
        """Energy and A = -beta E - log q_sym of the current configuration."""
        L = _lib()
        h = self.q._h
        _check(L.isg_learned_energies(h, _tptr(self.cur), 1, self.L, self.dim,
                                      _tptr(self.state), C.c_void_p(self.state.data_ptr() + 8)))
        lq = self.q.score(self.cur.view(1, -1))
        lqf = self.q.score(self.cur.view(1, -1), flip=True)
        _check(L.isg_learned_state_a(h, _tptr(lq), _tptr(lqf), _tptr(self.state), self.beta,
                                     self.J, _tptr(self.ax)))
        self.q.sync()  # lq/lqf are torch temporaries: finish before they are released

    def start(self, warm_sweeps: int = 200):
        self.ising.step(warm_sweeps)
        _check(_lib().isg_ising_store_natural(self.ising._h, 0, 0, _tptr(self.cur)))
        self._refresh_state()
        self.q.sync()

    def batch(self):
        """One round: sweeps, then K learned proposals; |M| per proposal recorded."""
        import torch
        L = _lib()
        h = self.q._h
        if self.next_sweeps > 0:
            _check(L.isg_ising_load_natural(self.ising._h, 0, 0, _tptr(self.cur)))
            self.ising.step(self.next_sweeps)
            _check(L.isg_ising_store_natural(self.ising._h, 0, 0, _tptr(self.cur)))
            self._refresh_state()
        props, lq, lqf = self.q.sample(self.K, 1 + self.step_no)
        _check(L.isg_learned_energies(h, _tptr(props), self.K, self.L, self.dim, _tptr(self.bond),
                                      _tptr(self.mag)))
        mrec = torch.empty(self.K, dtype=torch.int64, device=self.dev)
        brec = torch.empty(self.K, dtype=torch.int64, device=self.dev)
        _check(L.isg_learned_imh(h, _tptr(self.bond), _tptr(self.mag), _tptr(lq), _tptr(lqf),
                                 self.K, self.beta, self.J, _tptr(self.state), _tptr(self.ax),
                                 _tptr(mrec), _tptr(brec), _tptr(self.accepted),
                                 _tptr(self.work), 1 + self.step_no))
        _check(L.isg_learned_adopt(h, _tptr(props), _tptr(self.state), _tptr(self.cur)))
        self.q.sync()  # the library's stream: proposals and counters are complete
        self.records.append(mrec)
        self.brecords.append(brec)
        self.step_no += 1
        self.proposals += self.K
        acc = int(self.accepted.item())
        rate = (acc - self._acc_prev) / self.K
        self._acc_prev = acc
        self.batch_accept.append(rate)
        if self.step_no < self.burn_in:
            self.next_sweeps = self.fallback if rate < self.min_accept else self.sweeps
        elif self.step_no == self.burn_in:
            # frozen from here on: independent of the chain's later states
            mean = float(np.mean(self.batch_accept[:self.burn_in])) if self.burn_in else 1.0
            self.next_sweeps = self.fallback if mean < self.min_accept else self.sweeps
        return rate

    def m_series(self) -> np.ndarray:
        """|M| per site after every proposal."""
        import torch
        if not self.records:
            return np.zeros(0)
        return (torch.cat(self.records).double() / self.n).cpu().numpy()

    def e_series(self) -> np.ndarray:
        """Energy per site (-J bond / n) after every proposal."""
        import torch
        if not self.brecords:
            return np.zeros(0)
        return (-self.J * torch.cat(self.brecords).double() / self.n).cpu().numpy()


def collect_training_set(L: int, dim: int, T: float, chains: int = 64, rounds: int = 64,
                         gap: int = 20, warmup: int = 2000, seed: int = 3):
    """Configurations from the plain checkerboard sampler at temperature T:
    `chains` independent replicas, one snapshot every `gap` sweeps, with their
    negations (Z2).  Returns a torch int8 tensor (n, L^dim) on the GPU."""
    import torch
    b = IsingBatch([L], chains, seed=seed, dim=dim)
    b.set_temperatures([T] * chains)
    b.step(warmup)
    dev = torch.device("cuda", torch.cuda.current_device())
    n = L ** dim
    out = torch.empty((rounds * chains * 2, n), dtype=torch.int8, device=dev)
    k = 0
    for _ in range(rounds):
        b.step(gap)
        b.sync()
        for r in range(chains):
            _check(_lib().isg_ising_store_natural(b._h, 0, r, _tptr(out[k])))
            k += 1
    b.sync()
    out[k:] = -out[:k]
    perm = torch.randperm(out.shape[0], device=dev)
    return out[perm].contiguous()


class TrainingStream:
    """Fresh training configurations from the plain checkerboard sampler at
    temperature T: `chains` independent replicas advance `gap` sweeps between
    snapshots, so a network trained on the stream never sees a configuration
    twice.  next() returns the snapshot and its negations (Z2) as a torch
    int8 tensor (2 * chains, L^dim) on the GPU, in a shuffled order."""

    def __init__(self, L: int, dim: int, T: float, chains: int = 256, gap: int = 10,
                 warmup: int = 2000, seed: int = 3):
        import torch
        self.n = L ** dim
        self.chains, self.gap = int(chains), int(gap)
        self.b = IsingBatch([L], self.chains, seed=seed, dim=dim)
        self.b.set_temperatures([T] * self.chains)
        self.b.step(warmup)
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.buf = torch.empty((2 * self.chains, self.n), dtype=torch.int8, device=self.dev)
        self.gen = torch.Generator(device=self.dev)
        self.gen.manual_seed(seed)

    def next(self):
        import torch
        self.b.step(self.gap)
        _check(_lib().isg_ising_store_natural_all(self.b._h, 0, _tptr(self.buf)))
        self.b.sync()
        self.buf[self.chains:] = -self.buf[:self.chains]
        perm = torch.randperm(2 * self.chains, device=self.dev, generator=self.gen)
        return self.buf[perm].contiguous()

    def close(self):
        self.b.close()
