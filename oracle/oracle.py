"""ctypes bindings of the CPU oracle (oracle/isg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  Build it with
`make -C oracle` (done by __graft_entry__.build()).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB = None

i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def lib():
    global _LIB
    if _LIB is None:
        path = _HERE / "lib" / "liboracle.so"
        if not path.exists():
            raise RuntimeError(f"oracle not built: {path} missing (run `make -C oracle`)")
        L = C.CDLL(str(path))
        L.or_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.or_ising_thresholds.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, u32p]
        _bind_graph(L)
        _bind_cgraph(L)
        L.or_ising_hot_start.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_uint32, i8p]
        L.or_ising_halfsweep.argtypes = [C.c_int, C.c_int, i8p, C.c_int, C.c_uint64, C.c_uint32,
                                         C.c_uint64, u32p]
        L.or_ising_measure.argtypes = [C.c_int, C.c_int, i8p, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)]
        L.or_replica_uid.argtypes = [C.c_int, C.c_int]
        L.or_replica_uid.restype = C.c_uint32
        L.or_exchange_uid.argtypes = [C.c_int]
        L.or_exchange_uid.restype = C.c_uint32
        L.or_exchange.argtypes = [C.c_int, f64p, f64p, i32p, i32p, C.c_int, C.c_uint64, C.c_uint32,
                                  C.c_uint64]
        L.or_exchange.restype = C.c_int64
        L.or_ising_pt.argtypes = [C.c_int, C.c_int, C.c_int, i8p, f64p, C.c_double, C.c_double,
                                  C.c_uint64, i32p, i32p, u64p, u64p, u64p, i64p, C.c_int64,
                                  C.c_int64, C.c_int, C.c_int, i32p, i64p, i64p, C.c_int64]
        L.or_ising_pt.restype = C.c_int64
        L.or_ref_run.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                 C.c_int64, C.c_int64, f64p, f64p]
        L.or_replay_bench.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int64, C.c_int, C.c_uint64,
                                      C.POINTER(C.c_double)]
        L.or_replay_bench.restype = C.c_double
        L.or_jackknife.argtypes = [f64p, f64p, C.c_int64, C.c_double, C.c_double, C.c_int, f64p]
        L.or_refbench_create.argtypes = [i32p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                         C.c_uint64]
        L.or_refbench_create.restype = C.c_void_p
        L.or_refbench_step.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double)]
        L.or_refbench_step.restype = C.c_double
        L.or_refbench_destroy.argtypes = [C.c_void_p]
        if hasattr(L, "or_cont_hot_start"):
            _bind_cont(L)
        _LIB = L
    return _LIB


def _bind_cont(L):
    L.or_cont_hot_start.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_uint32, f64p]
    L.or_cont_overrelax.argtypes = [C.c_int, C.c_int, f64p, C.c_int, C.c_double]
    L.or_cont_metropolis.argtypes = [C.c_int, C.c_int, f64p, C.c_int, C.c_uint64, C.c_uint32,
                                     C.c_uint64, C.c_double, C.c_double, C.c_double,
                                     C.POINTER(C.c_int64)]
    L.or_cont_measure.argtypes = [C.c_int, C.c_int, f64p, f64p]
    L.or_cont_ref_sweep.argtypes = [C.c_int, f64p, C.c_double, C.c_double, C.c_double,
                                    C.c_uint64, C.c_uint64, C.c_int]


def cont_hot_start(L: int, nc: int, seed: int, r: int) -> np.ndarray:
    s = np.zeros(L ** 3 * nc, np.float64)
    lib().or_cont_hot_start(L, nc, seed, replica_uid(L, r), s)
    return s


def cont_overrelax(s: np.ndarray, L: int, nc: int, colour: int, J: float = 1.0) -> None:
    lib().or_cont_overrelax(L, nc, s, colour, J)


def cont_metropolis(s, L, nc, colour, seed, r, sweep, beta, J, delta) -> int:
    acc = C.c_int64(0)
    lib().or_cont_metropolis(L, nc, s, colour, seed, replica_uid(L, r), sweep, beta, J, delta,
                             C.byref(acc))
    return acc.value


def cont_measure(s: np.ndarray, L: int, nc: int) -> np.ndarray:
    out = np.zeros(10, np.float64)
    lib().or_cont_measure(L, nc, s, out)
    return out


def cont_ref_sweep(s, L, beta, J, delta, seed, sweep, n_or) -> None:
    lib().or_cont_ref_sweep(L, s, beta, J, delta, seed, sweep, n_or)


def nsites(L: int, dim: int = 3) -> int:
    return L ** dim


def philox(ctr, key) -> np.ndarray:
    out = np.zeros(4, np.uint32)
    lib().or_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def thresholds(dim: int, beta: float, J: float = 1.0, h: float = 0.0) -> np.ndarray:
    out = np.zeros(16, np.uint32)
    lib().or_ising_thresholds(dim, beta, J, h, out)
    return out


def replica_uid(L: int, r: int) -> int:
    return int(lib().or_replica_uid(L, r))


def hot_start(L: int, dim: int, seed: int, r: int) -> np.ndarray:
    s = np.zeros(nsites(L, dim), np.int8)
    lib().or_ising_hot_start(L, dim, seed, replica_uid(L, r), s)
    return s


def halfsweep(spins: np.ndarray, L: int, dim: int, colour: int, seed: int, r: int, sweep: int,
              thr: np.ndarray) -> None:
    lib().or_ising_halfsweep(L, dim, spins, colour, seed, replica_uid(L, r), sweep, thr)


def measure(spins: np.ndarray, L: int, dim: int = 3) -> tuple[int, int]:
    b, m = C.c_int64(), C.c_int64()
    lib().or_ising_measure(L, dim, spins, C.byref(b), C.byref(m))
    return b.value, m.value


class IsingPT:
    """Replay of one lattice size of the GPU PT protocol (bit-exact oracle)."""

    def __init__(self, L: int, dim: int, R: int, temps, seed: int, J: float = 1.0, h: float = 0.0):
        self.L, self.dim, self.R, self.seed, self.J, self.h = L, dim, R, seed, J, h
        self.temps = np.ascontiguousarray(temps, np.float64)
        self.spins = np.concatenate([hot_start(L, dim, seed, r) for r in range(R)])
        self.r2t = np.arange(R, dtype=np.int32)
        self.t2r = np.arange(R, dtype=np.int32)
        self.gsweep = np.zeros(1, np.uint64)
        self.ksample = np.zeros(1, np.uint64)
        self.xcount = np.zeros(1, np.uint64)
        self.accepted = np.zeros(1, np.int64)

    def replica_spins(self, r: int) -> np.ndarray:
        n = nsites(self.L, self.dim)
        return self.spins[r * n:(r + 1) * n]

    def warmup(self, n: int) -> None:
        z32 = np.zeros(1, np.int32)
        z64 = np.zeros(1, np.int64)
        lib().or_ising_pt(self.L, self.dim, self.R, self.spins, self.temps, self.J, self.h,
                          self.seed, self.r2t, self.t2r, self.gsweep, self.ksample, self.xcount,
                          self.accepted, n, 0, 1, 1, z32, z64, z64, 0)

    def reset_sampling(self) -> None:
        self.ksample[:] = 0
        self.xcount[:] = 0
        self.accepted[:] = 0

    def schedule(self, temps, n: int, measure_every: int = 0, measure_phase: int = 0):
        """isg_ising_run_schedule replayed: sweep k at temps[k] for every replica
        (temps None: current temperatures), no exchange; (bond, mag) records of shape
        (rows, R) after the sweeps with k % measure_every == measure_phase."""
        b, m = [], []
        for k in range(n):
            if temps is not None:
                self.temps[:] = temps[k]
            self.warmup(1)
            if measure_every > 0 and k % measure_every == measure_phase:
                bm = [measure(self.replica_spins(r), self.L, self.dim) for r in range(self.R)]
                b.append([x[0] for x in bm])
                m.append([x[1] for x in bm])
        return (np.array(b, np.int64).reshape(-1, self.R), np.array(m, np.int64).reshape(-1, self.R))

    def sample(self, n: int, exchange_every: int, measure_every: int):
        rows = n // measure_every + 2
        rt = np.zeros(rows * self.R, np.int32)
        rb = np.zeros(rows * self.R, np.int64)
        rm = np.zeros(rows * self.R, np.int64)
        got = lib().or_ising_pt(self.L, self.dim, self.R, self.spins, self.temps, self.J, self.h,
                                self.seed, self.r2t, self.t2r, self.gsweep, self.ksample,
                                self.xcount, self.accepted, 0, n, exchange_every, measure_every,
                                rt, rb, rm, rows)
        k = got * self.R
        return rt[:k].reshape(got, self.R), rb[:k].reshape(got, self.R), rm[:k].reshape(got, self.R)


def measure_observables(T: float, bond, mag, J: float, h: float, n3: float) -> list[float]:
    """LatticeGpu::measure (src/cuda/lattice_gpu.rs:205-251) restated: per-sample
    e = E/N with E = sum_i(-J s_i nb_i / 2 - h s_i) = -J*bond - h*M (exact for the
    integer sums), m = |M/N|, m_s = M/N; FP64 running sums in sample order;
    [T, <e>, <m>, <m^2>, <m^4>, Cv, chi] with chi from the signed m_s."""
    beta = 1.0 / T
    se = se2 = sm = sm2 = sm4 = sms = sms2 = 0.0
    for b, m in zip(np.asarray(bond).tolist(), np.asarray(mag).tolist()):
        e_per = (-J * float(b) - h * float(m)) / n3
        m_per = abs(float(m) / n3)
        m_signed = float(m) / n3
        se += e_per
        se2 += e_per * e_per
        sm += m_per
        sm2 += m_per * m_per
        sm4 += m_per * m_per * m_per * m_per
        sms += m_signed
        sms2 += m_signed * m_signed
    n = float(len(bond))
    ae, ae2, am, am2, am4, ams, ams2 = se / n, se2 / n, sm / n, sm2 / n, sm4 / n, sms / n, sms2 / n
    return [T, ae, am, am2, am4, beta * beta * (ae2 - ae * ae) * n3, beta * (ams2 - ams * ams) * n3]


def fss_anneal(sizes, dim: int, t_min: float, t_max: float, t_steps: int, J: float, h: float,
               warmup: int, samples: int, seed: int) -> np.ndarray:
    """The `fss --gpu` schedule (src/cuda/fss_gpu.rs:7-39) replayed on the GPU stream
    definition: per size one replica, temperatures from t_max down to t_min
    (T_k = t_min + (t_max - t_min)*k/(t_steps-1)), `warmup` sweeps then `samples`
    measured sweeps at each.  Returns [n_sizes, t_steps, 7] in ascending T."""
    out = np.zeros((len(sizes), t_steps, 7), np.float64)
    for i, L in enumerate(sizes):
        n3 = float(L ** dim)
        pt = IsingPT(L, dim, 1, [t_max], seed, J, h)
        for k in range(t_steps - 1, -1, -1):
            T = t_min + (t_max - t_min) * float(k) / float(t_steps - 1)
            pt.temps[:] = T
            pt.r2t[:] = 0
            pt.t2r[:] = 0
            pt.warmup(warmup)
            pt.reset_sampling()
            _, b, m = pt.sample(samples, samples + 1, 1)
            out[i, k] = measure_observables(T, b[:, 0], m[:, 0], J, h, n3)
    return out


def wall_density(bond: int, L: int) -> float:
    """domain_wall_density (src/cuda/lattice_gpu.rs:253-281) from the bond sum B of
    the 3 L^3 forward bonds: walls = (3 L^3 - B) / 2."""
    bonds = 3 * L ** 3
    return ((bonds - int(bond)) // 2) / bonds


def kz_sweep(n: int, J: float, t_start: float, t_end: float, taus, n_trials: int, warmup: int,
             freeze: int, freeze_t: float, base_seed: int) -> np.ndarray:
    """run_kz_sweep_gpu (src/cuda/kz_gpu.rs:46-95) replayed on the GPU stream
    definition: per tau_q a batch of n_trials replicas keyed by base_seed + tau_q,
    warm-up at t_start, the linear ramp of kibble_zurek.rs:78-84 floored at 0.01,
    optional freeze; [len(taus), 2] = mean and standard error of rho."""
    out = np.zeros((len(taus), 2))
    for i, tau in enumerate(taus):
        temps = [t_start] * warmup
        temps += [max(t_start + (t_end - t_start) * (float(k + 1) / float(tau)), 0.01)
                  for k in range(tau)]
        temps += [max(freeze_t, 0.01)] * freeze
        pt = IsingPT(n, 3, n_trials, [t_start] * n_trials, base_seed + tau, J, 0.0)
        pt.schedule(temps, len(temps))
        rho = [wall_density(measure(pt.replica_spins(r), n, 3)[0], n) for r in range(n_trials)]
        # plain left-to-right sums (Rust's Iterator::sum); Python's sum() of floats
        # is compensated and rounds differently
        acc = 0.0
        for x in rho:
            acc += x
        mean = acc / float(n_trials)
        err = 0.0
        if n_trials > 1:
            ss = 0.0
            for x in rho:
                ss += (x - mean) * (x - mean)
            var = ss / (float(n_trials) - 1.0)
            err = float(np.sqrt(var)) / float(np.sqrt(float(n_trials)))
        out[i] = (mean, err)
    return out


def coarsening(n: int, J: float, t_high: float, t_quench: float, warmup: int, steps: int,
               every: int, seed: int):
    """run_coarsening_gpu (src/cuda/coarsening_gpu.rs:6-31) replayed: (steps, rho)."""
    pt = IsingPT(n, 3, 1, [t_high], seed, J, 0.0)
    pt.warmup(warmup)
    pt.temps[:] = max(t_quench, 0.01)
    b, _ = pt.schedule(None, steps, every, 0)
    return (np.arange(len(b)) * every, np.array([wall_density(x, n) for x in b[:, 0]]))


def _bind_graph(L):
    L.or_graph_build.argtypes = [C.c_int, i32p, C.c_int, i32p, i32p, i32p]
    L.or_graph_build.restype = C.c_int
    L.or_graph_hot_start.argtypes = [C.c_int, C.c_int, C.c_uint64, u8p]
    L.or_graph_pt.argtypes = [C.c_int, i32p, C.c_int, C.c_int, u8p, f64p, C.c_double, C.c_uint64,
                              i32p, i32p, u64p, u64p, u64p, i64p, C.c_int64, C.c_int64, C.c_int,
                              C.c_int, i32p, i64p, i64p, C.c_int64]
    L.or_graph_pt.restype = C.c_int64
    L.or_graph_ref_pt.argtypes = [C.c_int, i32p, C.c_int, C.c_int, f64p, C.c_double, C.c_uint64,
                                  C.c_int64, C.c_int64, C.c_int, f64p]


def graph_colouring(n: int, edges) -> tuple[int, np.ndarray]:
    """Greedy proper colouring in node order (the device's): (classes, colour[n])."""
    e = np.ascontiguousarray(edges, np.int32).reshape(-1)
    rowptr = np.zeros(n + 1, np.int32)
    adj = np.zeros(max(len(e), 1), np.int32)
    col = np.zeros(n, np.int32)
    k = lib().or_graph_build(n, e, len(e) // 2, rowptr, adj, col)
    return k, col


class GraphPT:
    """Replay of the graph PT engine (isg_graph_*): bit-exact oracle."""

    def __init__(self, n: int, edges, R: int, temps, seed: int, J: float = 1.0):
        self.n, self.R, self.seed, self.J = n, R, seed, J
        self.edges = np.ascontiguousarray(edges, np.int32).reshape(-1)
        self.temps = np.ascontiguousarray(temps, np.float64)
        self.spins = np.zeros(n * R, np.uint8)
        lib().or_graph_hot_start(n, R, seed, self.spins)
        self.r2t = np.arange(R, dtype=np.int32)
        self.t2r = np.arange(R, dtype=np.int32)
        self.gsweep = np.zeros(1, np.uint64)
        self.ksample = np.zeros(1, np.uint64)
        self.xcount = np.zeros(1, np.uint64)
        self.accepted = np.zeros(1, np.int64)

    def _run(self, warm: int, samples: int, ee: int, me: int):
        rows = samples // me + 2
        rt = np.zeros(rows * self.R, np.int32)
        rb = np.zeros(rows * self.R, np.int64)
        rm = np.zeros(rows * self.R, np.int64)
        got = lib().or_graph_pt(self.n, self.edges, len(self.edges) // 2, self.R, self.spins,
                                self.temps, self.J, self.seed, self.r2t, self.t2r, self.gsweep,
                                self.ksample, self.xcount, self.accepted, warm, samples, ee, me,
                                rt, rb, rm, rows)
        k = got * self.R
        return rt[:k].reshape(got, self.R), rb[:k].reshape(got, self.R), rm[:k].reshape(got, self.R)

    def warmup(self, n: int) -> None:
        self._run(n, 0, 1, 1)

    def reset_sampling(self) -> None:
        self.ksample[:] = 0
        self.xcount[:] = 0
        self.accepted[:] = 0

    def sample(self, n: int, exchange_every: int, measure_every: int):
        return self._run(0, n, exchange_every, measure_every)

    def replica_spins(self, r: int) -> np.ndarray:
        d = self.spins[r * self.n:(r + 1) * self.n]
        return np.where(d == 1, -1, 1).astype(np.int8)


def graph_ref_pt(n: int, edges, temps, J: float, seed: int, warmup: int, samples: int,
                 ee: int) -> np.ndarray:
    """The reference's CPU algorithm on a graph (gpu_jfit.rs:172-262): per
    temperature [sum e, sum e^2, sum |m|, sum m^2, sum m^4, count]."""
    e = np.ascontiguousarray(edges, np.int32).reshape(-1)
    t = np.ascontiguousarray(temps, np.float64)
    out = np.zeros(6 * len(t), np.float64)
    lib().or_graph_ref_pt(n, e, len(e) // 2, len(t), t, J, seed, warmup, samples, ee, out)
    return out.reshape(len(t), 6)


def _bind_cgraph(L):
    L.or_cgraph_build.argtypes = [C.c_int, i32p, C.c_int, i32p, i32p, i32p]
    L.or_cgraph_build.restype = C.c_int
    L.or_cgraph_hot_start.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, f64p]
    L.or_cgraph_metro_sweep.argtypes = [C.c_int, i32p, i32p, i32p, C.c_int, f64p, C.c_uint32,
                                        C.c_uint64, C.c_uint64, C.c_double, C.c_double,
                                        C.c_double, C.POINTER(C.c_double)]
    L.or_cgraph_metro_sweep.restype = C.c_int64
    L.or_cgraph_wolff_sweep.argtypes = [C.c_int, i32p, i32p, f64p, C.c_uint32, C.c_uint64,
                                        C.c_uint64, C.c_double, C.c_double,
                                        C.POINTER(C.c_double)]
    L.or_cgraph_wolff_sweep.restype = C.c_int
    L.or_cgraph_measure.argtypes = [C.c_int, i32p, i32p, f64p, C.c_int, C.c_double,
                                    C.POINTER(C.c_double), f64p]
    L.or_cgraph_ref_pt.argtypes = [C.c_int, i32p, C.c_int, C.c_int, C.c_int, f64p, C.c_double,
                                   C.c_uint64, C.c_int64, C.c_int64, C.c_int, C.c_double, f64p]


class CGraphReplay:
    """Per-sweep FP64 replay of the continuous graph engine (isg_cgraph_*):
    hot start, one sweep of a replica (O(3) cone Metropolis by colour class,
    O(2) single-cluster Wolff), E and M.  `sweep` returns (moves, margin):
    accepted rotations or cluster size, and the smallest decision margin."""

    def __init__(self, n: int, edges, nc: int, seed: int):
        self.n, self.nc, self.seed = n, nc, seed
        e = np.ascontiguousarray(edges, np.int32).reshape(-1)
        self.rowptr = np.zeros(n + 1, np.int32)
        self.adj = np.zeros(max(len(e), 1), np.int32)
        self.colour = np.zeros(n, np.int32)
        self.ncol = lib().or_cgraph_build(n, e, len(e) // 2, self.rowptr, self.adj, self.colour)
        if self.ncol < 0:
            raise ValueError("bad graph")

    def hot_start(self, R: int) -> np.ndarray:
        out = np.zeros(R * self.n * self.nc, np.float64)
        lib().or_cgraph_hot_start(self.n, R, self.nc, self.seed, out)
        return out.reshape(R, self.n, self.nc)

    def sweep(self, sp: np.ndarray, replica: int, sweep: int, beta: float, J: float = 1.0,
              cos_delta: float | None = None):
        assert sp.dtype == np.float64 and sp.flags.c_contiguous and sp.size == self.n * self.nc
        margin = C.c_double(1e300)
        if self.nc == 3:
            cd = float(np.float32(np.cos(0.5))) if cos_delta is None else cos_delta
            mv = lib().or_cgraph_metro_sweep(self.n, self.rowptr, self.adj, self.colour, self.ncol,
                                             sp.reshape(-1), replica, self.seed, sweep, beta, J, cd,
                                             C.byref(margin))
        else:
            mv = lib().or_cgraph_wolff_sweep(self.n, self.rowptr, self.adj, sp.reshape(-1),
                                             replica, self.seed, sweep, beta, J, C.byref(margin))
        return int(mv), margin.value

    def measure(self, sp: np.ndarray, J: float = 1.0):
        e = C.c_double()
        m = np.zeros(self.nc, np.float64)
        lib().or_cgraph_measure(self.n, self.rowptr, self.adj,
                                np.ascontiguousarray(sp, np.float64).reshape(-1), self.nc, J,
                                C.byref(e), m)
        return e.value, m


def cgraph_ref_pt(n: int, edges, nc: int, temps, J: float, seed: int, warmup: int, samples: int,
                  ee: int, delta: float = 0.5) -> np.ndarray:
    """The reference's CPU algorithms on a graph (run_heisenberg_jfit for nc = 3,
    run_xy_jfit for nc = 2, gpu_jfit.rs:298-524): per temperature
    [sum e, sum e^2, sum |m|, sum m^2, sum m^4, count]."""
    e = np.ascontiguousarray(edges, np.int32).reshape(-1)
    t = np.ascontiguousarray(temps, np.float64)
    out = np.zeros(6 * len(t), np.float64)
    lib().or_cgraph_ref_pt(n, e, len(e) // 2, len(t), nc, t, J, seed, warmup, samples, ee, delta,
                           out)
    return out.reshape(len(t), 6)


def ref_run(L: int, dim: int, T: float, seed: int, warmup: int, samples: int, J=1.0, h=0.0):
    e = np.zeros(samples, np.float64)
    m = np.zeros(samples, np.float64)
    lib().or_ref_run(L, dim, T, J, h, seed, warmup, samples, e, m)
    return e, m


def replay_bench(L: int, dim: int, T: float, sweeps: int, threads: int, seed: int = 42):
    flips = C.c_double()
    sec = lib().or_replay_bench(L, dim, T, sweeps, threads, seed, C.byref(flips))
    return sec, flips.value


class RefBench:
    """Reference CPU path (random-site Metropolis) on `threads` host threads,
    each owning one replica of every size; step(sweeps) -> (seconds, flips)."""

    def __init__(self, sizes, dim, tmin, tmax, threads, seed=42):
        self.threads = threads
        self._h = lib().or_refbench_create(np.ascontiguousarray(sizes, np.int32), len(sizes), dim,
                                           tmin, tmax, threads, seed)

    def step(self, sweeps: float = 1.0):
        f = C.c_double()
        sec = lib().or_refbench_step(self._h, float(sweeps), C.byref(f))
        return sec, f.value

    def close(self):
        if self._h:
            lib().or_refbench_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def jackknife(e, m, beta: float, n3: float, n_blocks: int) -> np.ndarray:
    e = np.ascontiguousarray(e, np.float64)
    m = np.ascontiguousarray(m, np.float64)
    out = np.zeros(12, np.float64)
    lib().or_jackknife(e, m, len(e), beta, n3, n_blocks, out)
    return out


def exchange(betas, energies, r2t, t2r, parity: int, seed: int, L: int, xcount: int) -> int:
    return int(lib().or_exchange(len(betas), np.ascontiguousarray(betas, np.float64),
                                 np.ascontiguousarray(energies, np.float64), r2t, t2r, parity,
                                 seed, lib().or_exchange_uid(L), xcount))


# ---------------------------------------------------------------- numpy formulas
# Restated from analysis/scripts/reproduce_validation.py (reference).

def onsager_energy(T: float, J: float = 1.0) -> float:
    """reproduce_validation.py:71-77."""
    from scipy.special import ellipk
    k = J / T
    ek = 2 * np.sinh(2 * k) / np.cosh(2 * k) ** 2
    return float(-J * (1.0 / np.tanh(2 * k)) * (1 + (2 / np.pi) * (2 * np.tanh(2 * k) ** 2 - 1)
                                                 * ellipk(ek ** 2)))


def onsager_magnetization(T: float, J: float = 1.0) -> float:
    """reproduce_validation.py:80-85."""
    tc = 2 * J / np.log(1 + np.sqrt(2))
    if T >= tc:
        return 0.0
    k = J / T
    return float((1 - np.sinh(2 * k) ** (-4)) ** (1 / 8))


def exact_enumeration(L: int, dim: int, temps, J: float = 1.0) -> list[dict]:
    """All 2^(L^dim) states, periodic forward bonds; reproduce_validation.py:88-140
    (2D) generalised to a cubic lattice.  Returns E, M(|m|), M2, M4, Cv, chi_conn per T."""
    n = L ** dim
    states = np.arange(2 ** n, dtype=np.int64)
    spins = (((states[:, None] >> np.arange(n)) & 1) * 2 - 1).astype(np.int8)
    grid = spins.reshape((-1,) + (L,) * dim)
    bond = np.zeros(len(states), np.int64)
    for ax in range(1, dim + 1):
        bond += (grid * np.roll(grid, -1, axis=ax)).reshape(len(states), -1).sum(1)
    mag = spins.sum(1).astype(np.float64)
    energies = -J * bond.astype(np.float64)
    rows = []
    for T in temps:
        beta = 1.0 / T
        lw = -beta * energies
        w = np.exp(lw - lw.max())
        w /= w.sum()
        e = np.sum(w * energies) / n
        e2 = np.sum(w * energies ** 2) / n ** 2
        ma = np.sum(w * np.abs(mag)) / n
        m2 = np.sum(w * mag ** 2) / n ** 2
        m4 = np.sum(w * mag ** 4) / n ** 4
        rows.append(dict(T=T, E=e, M=ma, M2=m2, M4=m4, Cv=beta ** 2 * n * (e2 - e ** 2),
                         chi=beta * n * (m2 - ma ** 2)))
    return rows


def tau_int(x) -> float:
    """Windowed integrated autocorrelation time, reproduce_validation.py:143-163."""
    x = np.asarray(x, float)
    x = x - x.mean()
    n = len(x)
    max_lag = n // 4
    var = np.var(x)
    if var < 1e-15:
        return 0.5
    f = np.fft.rfft(x, 2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:max_lag]
    acf /= var * np.arange(n, n - max_lag, -1)
    tau = 0.5
    for t in range(1, len(acf)):
        tau += acf[t]
        if t >= 6 * tau:
            break
    return float(tau)


# --------------------------------------------------------------- reweighting
# numpy restatement of the reference's reweighting consumers: the checker of
# the device reweighting (isg_wham, isg_wham_weights, isg_reweight_single).


def _lse(x, axis=None):
    m = np.max(x, axis=axis, keepdims=True)
    out = m + np.log(np.sum(np.exp(x - m), axis=axis, keepdims=True))
    return np.squeeze(out, axis=axis) if axis is not None else float(out.reshape(()))


def rw_single_histogram(energies, beta_sim, beta_target):
    """analysis/scripts/reweighting.py:15-37: normalised exp(-(b' - b) E)."""
    lw = -(beta_target - beta_sim) * np.asarray(energies, np.float64)
    w = np.exp(lw - lw.max())
    return w / w.sum()


def _rw_wham_solve(energy_lists, beta_list, n_iter=100, tol=1e-8):
    """reweighting.py:69-95: the f_k iteration; returns (f, log_denom of the
    last round, all energies)."""
    b = np.asarray(beta_list, np.float64)
    nk = np.array([len(x) for x in energy_lists], np.float64)
    E = np.concatenate([np.asarray(x, np.float64) for x in energy_lists])
    f = np.zeros(len(b))
    ld = None
    for _ in range(n_iter):
        ld = _lse((np.log(nk) + f)[None, :] - b[None, :] * E[:, None], axis=1)
        fn = np.array([-_lse(-bk * E - ld) for bk in b])
        fn -= fn[0]
        done = np.max(np.abs(fn - f)) < tol
        f = fn
        if done:
            break
    return f, ld, E


def rw_wham(energy_lists, beta_list, beta_target, n_iter=100, tol=1e-8):
    """reweighting.py:45-105: (normalised weights, simulation index)."""
    _, ld, E = _rw_wham_solve(energy_lists, beta_list, n_iter, tol)
    lw = -beta_target * E - ld
    w = np.exp(lw - lw.max())
    w /= w.sum()
    sim = np.concatenate([np.full(len(x), k) for k, x in enumerate(energy_lists)])
    return w, sim


def rw_binder(energy_lists, mag_lists, beta_list, beta_targets):
    """reweighting.py:108-143: (T, U) with U = 1 - <m^4> / (3 <m^2>^2)."""
    m = np.concatenate([np.asarray(x, np.float64) for x in mag_lists])
    T, U = [], []
    for bt in beta_targets:
        w, _ = rw_wham(energy_lists, beta_list, bt)
        m2 = np.sum(w * m ** 2)
        m4 = np.sum(w * m ** 4)
        T.append(1.0 / bt)
        U.append(1.0 - m4 / (3.0 * m2 ** 2) if m2 > 0 else 0.0)
    return np.array(T), np.array(U)


def _rw_fine_row(T, beta_t, V, w, e, m, e_sim, m_sim, db):
    """Observables of one target (analyze_gpu_fss.py:103-155 / 218-241):
    averages from weights w over (e, m); errors from the leave-one-block-out
    single-histogram jackknife (20 blocks) of the closest simulation."""
    am, am2, am4 = w @ m, w @ m ** 2, w @ m ** 4
    ae, ae2 = w @ e, w @ e ** 2
    chi = beta_t * V * (am2 - am ** 2)
    cv = beta_t ** 2 * (ae2 - ae ** 2) / V
    U = 1.0 - am4 / (3.0 * am2 ** 2) if am2 > 1e-15 else 0.0
    nb = 20
    bs = len(e_sim) // nb
    jc, jm, ju = np.zeros(nb), np.zeros(nb), np.zeros(nb)
    for k in range(nb):
        idx = np.concatenate([np.arange(0, k * bs), np.arange((k + 1) * bs, nb * bs)])
        ej, mj = e_sim[idx], m_sim[idx]
        lw = -db * ej
        wj = np.exp(lw - lw.max())
        wj /= wj.sum()
        j1, j2, j4 = np.sum(wj * mj), np.sum(wj * mj ** 2), np.sum(wj * mj ** 4)
        jc[k] = beta_t * V * (j2 - j1 ** 2)
        jm[k] = j1
        ju[k] = 1.0 - j4 / (3.0 * j2 ** 2) if j2 > 1e-15 else 0.0
    f = (nb - 1.0) / nb
    return {"T": T, "M": am, "M2": am2, "M4": am4, "chi_conn": chi,
            "chi_err": np.sqrt(f * np.sum((jc - chi) ** 2)), "Cv": cv, "U": U, "E": ae / V,
            "M_err": np.sqrt(f * np.sum((jm - am) ** 2)),
            "U_err": np.sqrt(f * np.sum((ju - U) ** 2))}


def _rw_table(rows):
    return {k: np.array([r[k] for r in rows]) for k in rows[0]}


def rw_single_fine(energy_lists, mag_lists, beta_list, T_fine, n):
    """analyze_gpu_fss.py:86-157: single-histogram reweighting of the closest
    simulation to every T of a fine grid (energies are totals, V = n^3)."""
    V = n ** 3
    b = np.asarray(beta_list, np.float64)
    rows = []
    for T in T_fine:
        bt = 1.0 / T
        k = int(np.argmin(np.abs(1.0 / b - T)))
        e = np.asarray(energy_lists[k], np.float64)
        m = np.asarray(mag_lists[k], np.float64)
        w = rw_single_histogram(e, b[k], bt)
        rows.append(_rw_fine_row(T, bt, V, w, e, m, e, m, bt - b[k]))
    return _rw_table(rows)


def rw_wham_fine(energy_lists, mag_lists, beta_list, T_fine, n, n_iter=100, tol=1e-8):
    """analyze_gpu_fss.py:160-243: WHAM over all simulations at every T of a
    fine grid, errors from the closest simulation's single-histogram jackknife."""
    V = n ** 3
    b = np.asarray(beta_list, np.float64)
    _, ld, E = _rw_wham_solve(energy_lists, b, n_iter, tol)
    M = np.concatenate([np.asarray(x, np.float64) for x in mag_lists])
    rows = []
    for T in T_fine:
        bt = 1.0 / T
        lw = -bt * E - ld
        w = np.exp(lw - lw.max())
        w /= w.sum()
        k = int(np.argmin(np.abs(1.0 / b - T)))
        e_sim = np.asarray(energy_lists[k], np.float64)
        m_sim = np.asarray(mag_lists[k], np.float64)
        rows.append(_rw_fine_row(T, bt, V, w, E, M, e_sim, m_sim, bt - b[k]))
    return _rw_table(rows)
