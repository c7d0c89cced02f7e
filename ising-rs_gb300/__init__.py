"""ising-rs_gb300 — Python host mirror of the reference's GPU backend interface.

Thin ctypes layer over libisinggb (include/isg.h), the sm_103a engine.  It
mirrors the names, argument meaning and error behaviour of faulknco/ising-rs's
backend for the checkerboard PT path:

  LatticeGpu            src/cuda/lattice_gpu.rs:9-189  (new/step/warm_up/
                        measure_gpu/energy_gpu/get_spins)
  ContinuousGpuLattice  src/cuda/gpu_lattice_continuous.rs:9-245
  linspace_temperatures src/parallel_tempering.rs:39-46
  jackknife_observables src/bin/gpu_fss.rs:327-412
  FssConfig, Observables, run_fss_gpu
                        src/fss.rs:6-36, src/observables.rs:5-13,
                        src/cuda/fss_gpu.rs:7-39 (annealing `fss --gpu`)
  KzProtocol, KzSweepPoint, run_kz_sweep_gpu
                        src/kibble_zurek.rs:11-76, src/cuda/kz_gpu.rs:46-95
  CoarseningConfig, CoarseningPoint, run_coarsening_gpu
                        src/coarsening.rs:14-56, src/cuda/coarsening_gpu.rs:6-31
  GraphDef              src/graph.rs:4-79 (JSON / edge-CSV readers) with BCC,
                        FCC and diluted-cubic builders
  GraphBatch            Ising PT on a graph (src/bin/gpu_jfit.rs:172-297)
  ContinuousGraphBatch  Heisenberg / XY PT on a graph (gpu_jfit.rs:298-524)
  single_histogram, reweight_observable, wham_reweight, reweight_binder
                        analysis/scripts/reweighting.py:15-143 (on the GPU)
  reweight_single_histogram, wham_reweight_fine
                        analysis/scripts/analyze_gpu_fss.py:86-243
  IsingBatch.hist_*, wham_histograms, read/write_timeseries, read_histograms
                        device energy histograms and the binary files of the
                        PT timeseries (include/isg.h)
  IsingBatch / ContinuousBatch: every (size, replica) lattice of a run in one
  handle (the GB300 replacement of the reference's Vec<LatticeGpu>).

Every failure raises IsingError (the reference returns anyhow::Result and its
drivers panic).  There is no CPU fallback: if the compiled library is missing
the import of any class fails loudly.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
_LIB = None

ISG_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "device timeout", -4: "unsupported",
          -5: "bad call order"}


class IsingError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{ERRORS.get(status, 'error')} ({status}): {message}")
        self.status = status


def library_path() -> Path:
    return _PKG / "lib" / "libisinggb.so"


def lib():
    """Load libisinggb; raises if it has not been built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        raise IsingError(-4, f"{path} not built; run python ising-rs_gb300/build.py")
    L = C.CDLL(str(path))
    _declare(L)
    _LIB = L
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _declare(L):
    vp, i32, i64, u64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double
    L.isg_last_error.restype = C.c_char_p
    L.isg_version.restype = i32
    sig = {
        "isg_ising_create": [C.POINTER(vp), vp, i32, i32, i32, u64],
        "isg_ising_destroy": [vp],
        "isg_ising_set_stream": [vp, vp],
        "isg_ising_set_temperatures": [vp, vp, dbl, dbl],
        "isg_ising_step": [vp, i64],
        "isg_ising_measure": [vp, vp, vp],
        "isg_ising_exchange": [vp, i32, vp],
        "isg_ising_get_r2t": [vp, vp],
        "isg_ising_set_r2t": [vp, vp],
        "isg_ising_get_spins": [vp, i32, i32, vp],
        "isg_ising_set_spins": [vp, i32, i32, vp],
        "isg_ising_pt_run": [vp, i64, i32, i32, vp, vp, vp, i64, vp],
        "isg_ising_run_schedule": [vp, vp, i64, i32, i32, vp, vp, i64, vp],
        "isg_ising_read_records": [vp, vp, vp, vp, i64, vp],
        "isg_ising_reset_sampling": [vp],
        "isg_ising_get_accepted": [vp, vp],
        "isg_ising_get_sweep": [vp, vp],
        "isg_ising_sync": [vp],
        "isg_ising_set_launch": [vp, i32, i32],
        "isg_ising_autotune": [vp, vp],
        "isg_ising_set_prefetch": [vp, i32],
        "isg_ising_set_cache_prefetch": [vp, i32, i32],
        "isg_ising_set_words_per_lane": [vp, i32],
        "isg_ising_set_dependent_launch": [vp, i32],
        "isg_ising_set_resident_pt": [vp, i32],
        "isg_ising_time_halfsweep": [vp, i32, vp],
        "isg_ising_time_halfsweep_graph": [vp, i32, i64, i32, vp],
        "isg_ising_sites_per_halfsweep": [vp, vp],
        "isg_jackknife": [vp, vp, i64, dbl, dbl, i32, vp],
        "isg_fss_anneal": [vp, i32, i32, dbl, dbl, i32, dbl, dbl, i64, i64, u64, vp],
        "isg_kz_sweep": [i32, dbl, dbl, dbl, vp, i32, i32, i64, i64, dbl, u64, vp],
        "isg_graph_create": [C.POINTER(vp), i32, vp, i32, i32, u64],
        "isg_graph_destroy": [vp],
        "isg_graph_num_colours": [vp, vp],
        "isg_graph_set_temperatures": [vp, vp, dbl],
        "isg_graph_step": [vp, i64],
        "isg_graph_reset_sampling": [vp],
        "isg_graph_pt_run": [vp, i64, i32, i32, vp, vp, vp, i64, vp],
        "isg_graph_get_accepted": [vp, vp],
        "isg_graph_get_spins": [vp, i32, vp],
        "isg_graph_get_r2t": [vp, vp],
        "isg_barrier_selftest": [i32, i32, i64, vp],
        "isg_cgraph_create": [C.POINTER(vp), i32, vp, i32, i32, i32, u64],
        "isg_cgraph_destroy": [vp],
        "isg_cgraph_num_colours": [vp, vp],
        "isg_cgraph_set_temperatures": [vp, vp, dbl],
        "isg_cgraph_set_delta": [vp, dbl],
        "isg_cgraph_step": [vp, i64],
        "isg_cgraph_reset_sampling": [vp],
        "isg_cgraph_pt_run": [vp, i64, i32, i32, vp, vp, vp, i64, vp],
        "isg_cgraph_get_accepted": [vp, vp],
        "isg_cgraph_get_moves": [vp, vp],
        "isg_cgraph_get_spins": [vp, i32, vp],
        "isg_cgraph_set_spins": [vp, i32, vp],
        "isg_cgraph_get_r2t": [vp, vp],
        "isg_cgraph_get_sweep": [vp, vp],
        "isg_coarsening": [i32, dbl, dbl, dbl, i64, i64, i64, u64, vp, vp, i64, vp],
        "isg_ising_hist_enable": [vp, i32],
        "isg_ising_hist_reset": [vp],
        "isg_ising_hist_range": [vp, i32, i32, vp, vp],
        "isg_ising_hist_read": [vp, i32, i32, i64, i64, vp],
        "isg_wham": [vp, vp, vp, i32, i64, vp, vp, i32, i32, dbl, vp, i32, vp, vp, vp],
        "isg_wham_weights": [vp, vp, i64, vp, vp, i32, i32, dbl, dbl, vp, vp, vp],
        "isg_reweight_single": [vp, vp, vp, i32, i64, vp, vp, vp, vp, vp, vp, i32, vp],
        "isg_ts_open": [C.POINTER(vp), C.c_char_p, i32, i32, vp, i32],
        "isg_ts_append": [vp, vp, vp, vp, vp, i64],
        "isg_ts_close": [vp],
        "isg_hist_write": [C.c_char_p, i32, i32, dbl, vp, i32, vp, vp, vp],
        "isg_cont_create": [C.POINTER(vp), vp, i32, i32, i32, u64],
        "isg_cont_destroy": [vp],
        "isg_cont_set_stream": [vp, vp],
        "isg_cont_set_temperatures": [vp, vp, dbl],
        "isg_cont_sweep": [vp, i64, dbl, i32],
        "isg_cont_overrelax": [vp, i32],
        "isg_cont_metropolis": [vp, i32, dbl],
        "isg_cont_normalize": [vp],
        "isg_cont_measure": [vp, vp, vp, vp],
        "isg_cont_exchange": [vp, i32, vp],
        "isg_cont_pt_run": [vp, i64, i32, i32, dbl, i32, i32, vp, vp, vp, vp, i64, vp],
        "isg_cont_reset_sampling": [vp],
        "isg_cont_get_r2t": [vp, vp],
        "isg_cont_get_spins": [vp, i32, i32, vp],
        "isg_cont_set_spins": [vp, i32, i32, vp],
        "isg_cont_get_accepted": [vp, vp],
        "isg_cont_get_metro_accepted": [vp, vp],
        "isg_cont_sync": [vp],
        "isg_cont_time_kernels": [vp, i32, vp],
        "isg_cont_set_fused_measure": [vp, i32],
        "isg_cont_sites_per_sweep": [vp, vp],
    }
    for name, args in sig.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = i32


def _check(status: int) -> None:
    if status != ISG_OK:
        raise IsingError(status, lib().isg_last_error().decode(errors="replace"))


def linspace_temperatures(t_min: float, t_max: float, n: int) -> list[float]:
    """src/parallel_tempering.rs:39-46 (same FP64 expression)."""
    if n == 1:
        return [t_min]
    return [t_min + (t_max - t_min) * i / (n - 1) for i in range(n)]


def jackknife_observables(e, m, beta: float, n3: float, n_blocks: int) -> np.ndarray:
    """src/bin/gpu_fss.rs:327-412 via isg_jackknife: [E, E_err, M, M_err, M2, M2_err,
    M4, M4_err, Cv, Cv_err, chi, chi_err]."""
    e = np.ascontiguousarray(e, np.float64)
    m = np.ascontiguousarray(m, np.float64)
    out = np.zeros(12, np.float64)
    _check(lib().isg_jackknife(_ptr(e), _ptr(m), len(e), beta, n3, n_blocks, _ptr(out)))
    return out


def binder(m2: float, m4: float) -> float:
    """U4 = 1 - <m^4> / (3 <m^2>^2) (analysis/scripts/ising_stats.py:66)."""
    if m2 <= 1e-15:
        return 0.0
    return 1.0 - m4 / (3.0 * m2 * m2)


@dataclass
class Observables:
    """src/observables.rs:5-13: per-spin averages at one temperature."""
    temperature: float
    energy: float
    magnetisation: float
    heat_capacity: float
    susceptibility: float
    m2: float
    m4: float


def _observables(temperature: float, bond, mag, J: float, h: float, n3: float) -> Observables:
    """Per-temperature statistics of LatticeGpu::measure (src/cuda/lattice_gpu.rs:205-251),
    operation for operation in FP64, from per-sweep integer bond and magnetisation sums."""
    beta = 1.0 / temperature
    se = se2 = sm = sm2 = sm4 = sms = sms2 = 0.0
    for b, m in zip(bond.tolist(), mag.tolist()):
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
    s = float(len(bond))
    ae, ae2, am, am2, am4, ams, ams2 = se / s, se2 / s, sm / s, sm2 / s, sm4 / s, sms / s, sms2 / s
    return Observables(temperature, ae, am, beta * beta * (ae2 - ae * ae) * n3,
                       beta * (ams2 - ams * ams) * n3, am2, am4)


@dataclass
class FssConfig:
    """src/fss.rs:6-36 (FssConfig and its Default).  The GPU path is cubic Metropolis;
    `geometry` and `algorithm` are kept for interface parity and not used by it."""
    sizes: list = field(default_factory=lambda: [8, 12, 16, 20, 24, 28])
    geometry: str = "cubic"
    j: float = 1.0
    h: float = 0.0
    t_min: float = 3.5
    t_max: float = 5.5
    t_steps: int = 41
    warmup_sweeps: int = 500
    sample_sweeps: int = 200
    seed: int = 42
    algorithm: str = "wolff"


def run_fss_gpu(config: FssConfig, dim: int = 3) -> list:
    """src/cuda/fss_gpu.rs:7-39 through isg_fss_anneal: for every size, anneal from
    t_max down to t_min; returns [(n, [Observables in ascending T])]."""
    sizes = [int(n) for n in config.sizes]
    if not sizes:
        return []
    ts = int(config.t_steps)
    out = np.zeros((len(sizes), ts, 7), np.float64)
    sz = np.ascontiguousarray(sizes, np.int32)
    _check(lib().isg_fss_anneal(_ptr(sz), len(sizes), int(dim), float(config.t_min),
                                float(config.t_max), ts, float(config.j), float(config.h),
                                int(config.warmup_sweeps), int(config.sample_sweeps),
                                int(config.seed), _ptr(out)))
    def obs(r):  # library row order: T, E, M, M2, M4, Cv, chi
        return Observables(temperature=float(r[0]), energy=float(r[1]),
                           magnetisation=float(r[2]), heat_capacity=float(r[5]),
                           susceptibility=float(r[6]), m2=float(r[3]), m4=float(r[4]))
    return [(n, [obs(out[i, k]) for k in range(ts)]) for i, n in enumerate(sizes)]


@dataclass
class KzProtocol:
    """src/kibble_zurek.rs:11-34."""
    warmup_sweeps: int = 200
    freeze_sweeps: int = 0
    freeze_temperature: float = 0.01

    def describe(self) -> str:
        return (f"warmup={self.warmup_sweeps} sweeps, ramp endpoint measurement, "
                f"freeze={self.freeze_sweeps} sweeps at T={self.freeze_temperature:.4f}")


@dataclass
class KzSweepPoint:
    """src/kibble_zurek.rs:63-69."""
    tau_q: int
    rho: float
    rho_err: float
    n_trials: int


def run_kz_sweep_gpu(n: int, geometry: str, j: float, t_start: float, t_end: float,
                     tau_q_values, n_trials: int, protocol: KzProtocol | None = None,
                     base_seed: int = 42) -> list:
    """src/cuda/kz_gpu.rs:46-95 through isg_kz_sweep (cubic only, as the reference)."""
    if geometry not in ("cubic", "Cubic3D"):
        raise IsingError(-4, "GPU KZ only supports cubic geometry")
    protocol = protocol or KzProtocol()
    taus = np.ascontiguousarray([int(t) for t in tau_q_values], np.int64)
    if len(taus) == 0:
        return []
    out = np.zeros((len(taus), 2), np.float64)
    _check(lib().isg_kz_sweep(int(n), float(j), float(t_start), float(t_end), _ptr(taus),
                              len(taus), int(n_trials), int(protocol.warmup_sweeps),
                              int(protocol.freeze_sweeps), float(protocol.freeze_temperature),
                              int(base_seed), _ptr(out)))
    return [KzSweepPoint(int(t), float(r), float(e), int(n_trials))
            for t, (r, e) in zip(taus.tolist(), out)]


@dataclass
class CoarseningConfig:
    """src/coarsening.rs:14-50 (CoarseningConfig and its Default)."""
    n: int = 30
    geometry: str = "cubic"
    j: float = 1.0
    t_high: float = 10.0
    t_quench: float = 0.5
    warmup_sweeps: int = 200
    total_steps: int = 50_000
    sample_every: int = 100
    seed: int = 42


@dataclass
class CoarseningPoint:
    """src/coarsening.rs:52-56."""
    step: int
    rho: float


def run_coarsening_gpu(config: CoarseningConfig) -> list:
    """src/cuda/coarsening_gpu.rs:6-31 through isg_coarsening (cubic lattice)."""
    pts = (int(config.total_steps) - 1) // int(config.sample_every) + 1 \
        if config.total_steps > 0 and config.sample_every > 0 else 0
    st = np.zeros(max(pts, 1), np.int64)
    rho = np.zeros(max(pts, 1), np.float64)
    n = C.c_int64()
    _check(lib().isg_coarsening(int(config.n), float(config.j), float(config.t_high),
                                float(config.t_quench), int(config.warmup_sweeps),
                                int(config.total_steps), int(config.sample_every), int(config.seed),
                                _ptr(st), _ptr(rho), pts, C.byref(n)))
    return [CoarseningPoint(int(a), float(b)) for a, b in zip(st[:n.value], rho[:n.value])]


def _stream_handle(stream) -> int | None:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return int(stream.cuda_stream)
    return int(stream)


class IsingBatch:
    """Every (size, replica) int8 Ising lattice of a run on one GPU."""

    def __init__(self, sizes, replicas: int, seed: int = 42, dim: int = 3):
        self.sizes = [int(s) for s in sizes]
        self.replicas = int(replicas)
        self.dim = int(dim)
        self.seed = int(seed)
        arr = np.ascontiguousarray(self.sizes, np.int32)
        h = C.c_void_p()
        _check(lib().isg_ising_create(C.byref(h), _ptr(arr), len(self.sizes), self.replicas,
                                      self.dim, self.seed))
        self._h = h
        self.temps = None

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().isg_ising_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_total(self) -> int:
        return len(self.sizes) * self.replicas

    def nsites(self, s: int) -> int:
        return self.sizes[s] ** self.dim

    def set_stream(self, stream) -> None:
        h = _stream_handle(stream)
        _check(lib().isg_ising_set_stream(self._h, C.c_void_p(h) if h else None))

    def set_temperatures(self, temps, J: float = 1.0, h: float = 0.0) -> None:
        t = np.asarray(temps, np.float64)
        if t.ndim == 1 and len(t) == self.replicas:
            t = np.tile(t, len(self.sizes))
        t = np.ascontiguousarray(t.reshape(-1), np.float64)
        if len(t) != self.n_total:
            raise IsingError(-1, "need one temperature per (size, slot)")
        _check(lib().isg_ising_set_temperatures(self._h, _ptr(t), float(J), float(h)))
        self.temps = t.reshape(len(self.sizes), self.replicas)
        self.J, self.h = float(J), float(h)

    def step(self, n_sweeps: int = 1) -> None:
        _check(lib().isg_ising_step(self._h, int(n_sweeps)))

    def measure(self) -> tuple[np.ndarray, np.ndarray]:
        b = np.zeros(self.n_total, np.int64)
        m = np.zeros(self.n_total, np.int64)
        _check(lib().isg_ising_measure(self._h, _ptr(b), _ptr(m)))
        return b, m

    def exchange(self, parity: int = -1) -> np.ndarray:
        acc = np.zeros(len(self.sizes), np.int64)
        _check(lib().isg_ising_exchange(self._h, int(parity), _ptr(acc)))
        return acc

    def r2t(self) -> np.ndarray:
        out = np.zeros(self.n_total, np.int32)
        _check(lib().isg_ising_get_r2t(self._h, _ptr(out)))
        return out

    def set_r2t(self, r2t) -> None:
        a = np.ascontiguousarray(r2t, np.int32)
        _check(lib().isg_ising_set_r2t(self._h, _ptr(a)))

    def get_spins(self, s: int, r: int) -> np.ndarray:
        out = np.zeros(self.nsites(s), np.int8)
        _check(lib().isg_ising_get_spins(self._h, s, r, _ptr(out)))
        return out

    def set_spins(self, s: int, r: int, spins) -> None:
        a = np.ascontiguousarray(spins, np.int8).reshape(-1)
        if len(a) != self.nsites(s):
            raise IsingError(-1, "wrong number of spins")
        _check(lib().isg_ising_set_spins(self._h, s, r, _ptr(a)))

    def reset_sampling(self) -> None:
        _check(lib().isg_ising_reset_sampling(self._h))

    def pt_run(self, n_sweeps: int, exchange_every: int, measure_every: int):
        """Returns (slot, bond, mag) arrays of shape (records, n_total)."""
        rows = n_sweeps // measure_every + 1
        t = np.zeros((rows, self.n_total), np.int32)
        b = np.zeros((rows, self.n_total), np.int64)
        m = np.zeros((rows, self.n_total), np.int64)
        n = C.c_int64()
        _check(lib().isg_ising_pt_run(self._h, int(n_sweeps), int(exchange_every),
                                      int(measure_every), _ptr(t), _ptr(b), _ptr(m), rows,
                                      C.byref(n)))
        k = n.value
        return t[:k], b[:k], m[:k]

    def run_schedule(self, temps=None, n_sweeps: int | None = None, measure_every: int = 0,
                     measure_phase: int = 0):
        """Sweep k at temps[k] for every lattice (temps None: current temperatures,
        n_sweeps sweeps); returns (bond, mag) records of shape (rows, n_total) for the
        sweeps with k % measure_every == measure_phase."""
        if temps is not None:
            t = np.ascontiguousarray(temps, np.float64)
            n_sweeps = len(t) if n_sweeps is None else int(n_sweeps)
            if len(t) < n_sweeps:
                raise IsingError(-1, "need one temperature per sweep")
            tp = _ptr(t)
        else:
            tp = None
        n_sweeps = int(n_sweeps or 0)
        rows = 0
        if measure_every > 0 and n_sweeps > measure_phase:
            rows = (n_sweeps - 1 - measure_phase) // measure_every + 1
        b = np.zeros((max(rows, 1), self.n_total), np.int64)
        m = np.zeros((max(rows, 1), self.n_total), np.int64)
        n = C.c_int64()
        _check(lib().isg_ising_run_schedule(self._h, tp, n_sweeps, int(measure_every),
                                            int(measure_phase), _ptr(b), _ptr(m), rows,
                                            C.byref(n)))
        if temps is not None:
            self.temps = np.full((len(self.sizes), self.replicas), float(t[n_sweeps - 1]))
        return b[:n.value], m[:n.value]

    def pt_launch(self, n_sweeps: int, exchange_every: int, measure_every: int) -> None:
        """Asynchronous PT sweeps; records stay on the device (read_records)."""
        _check(lib().isg_ising_pt_run(self._h, int(n_sweeps), int(exchange_every),
                                      int(measure_every), None, None, None, 0, None))

    def read_records(self, max_records: int):
        t = np.zeros((max_records, self.n_total), np.int32)
        b = np.zeros((max_records, self.n_total), np.int64)
        m = np.zeros((max_records, self.n_total), np.int64)
        n = C.c_int64()
        _check(lib().isg_ising_read_records(self._h, _ptr(t), _ptr(b), _ptr(m), int(max_records),
                                            C.byref(n)))
        k = n.value
        return t[:k], b[:k], m[:k]

    def accepted(self) -> np.ndarray:
        out = np.zeros(len(self.sizes), np.int64)
        _check(lib().isg_ising_get_accepted(self._h, _ptr(out)))
        return out

    def sweep_counter(self) -> int:
        v = C.c_uint64()
        _check(lib().isg_ising_get_sweep(self._h, C.byref(v)))
        return v.value

    def sync(self) -> None:
        _check(lib().isg_ising_sync(self._h))

    def hist_enable(self, enable: bool = True) -> None:
        """Exact energy histograms of every (size, slot), accumulated by each
        record of pt_run: bins of the bond sum with the sums of |m|, m^2, m^4."""
        _check(lib().isg_ising_hist_enable(self._h, int(bool(enable))))

    def hist_reset(self) -> None:
        _check(lib().isg_ising_hist_reset(self._h))

    def histogram(self, size_index: int, slot: int):
        """(bond sums, counters (n, 4) uint64) of the visited bins of (size,
        slot): samples and the sums of |m|, m^2, m^4 in units of 2^-32."""
        lo, nb = C.c_int64(), C.c_int64()
        _check(lib().isg_ising_hist_range(self._h, int(size_index), int(slot), C.byref(lo),
                                          C.byref(nb)))
        out = np.zeros((nb.value, 4), np.uint64)
        if nb.value:
            _check(lib().isg_ising_hist_read(self._h, int(size_index), int(slot), lo.value,
                                             nb.value, _ptr(out)))
        return lo.value + 4 * np.arange(nb.value, dtype=np.int64), out

    def set_launch(self, threads: int, blocks_per_sm: int = 0) -> None:
        _check(lib().isg_ising_set_launch(self._h, threads, blocks_per_sm))

    def set_prefetch(self, depth: int = 0) -> None:
        """Rolling prefetch depth 1 or 2 (0 = automatic); results never depend on it."""
        _check(lib().isg_ising_set_prefetch(self._h, int(depth)))

    def set_cache_prefetch(self, level: int = 2, planes: int = 0) -> None:
        """Rolling half-sweep: prefetch `planes` z-planes ahead into L1 (level 1)
        or L2 (level 2); 0 planes = off."""
        _check(lib().isg_ising_set_cache_prefetch(self._h, int(level), int(planes)))

    def set_words_per_lane(self, words: int = 4) -> None:
        """Rolling half-sweep, L >= 128: 4 or 2 words per lane (same results)."""
        _check(lib().isg_ising_set_words_per_lane(self._h, int(words)))

    def set_resident_pt(self, enable: bool = True) -> None:
        """pt_run of small lattices in one cooperative resident launch (same bits)."""
        _check(lib().isg_ising_set_resident_pt(self._h, int(bool(enable))))

    def set_dependent_launch(self, enable: bool = True) -> None:
        """Half-sweep word kernels as programmatic dependent launches (same results)."""
        _check(lib().isg_ising_set_dependent_launch(self._h, int(bool(enable))))

    def autotune(self) -> tuple[int, int, int]:
        """Fastest (site threads, blocks per SM, prefetch depth), kept for the batch."""
        best = np.zeros(3, np.int32)
        _check(lib().isg_ising_autotune(self._h, _ptr(best)))
        return int(best[0]), int(best[1]), int(best[2])

    def time_halfsweep(self, n_launches: int = 20) -> float:
        v = C.c_float()
        _check(lib().isg_ising_time_halfsweep(self._h, n_launches, C.byref(v)))
        return v.value

    def time_halfsweep_graph(self, n_launches: int = 20, flush_bytes: int = 256 << 20,
                             replays: int = 5) -> float:
        """Mean ms of one half-sweep inside a captured graph of n_launches
        half-sweeps, L2 flushed before each replay (as in a timed PT step)."""
        v = C.c_float()
        _check(lib().isg_ising_time_halfsweep_graph(self._h, n_launches, int(flush_bytes),
                                                    replays, C.byref(v)))
        return v.value

    def sites_per_halfsweep(self) -> int:
        v = C.c_int64()
        _check(lib().isg_ising_sites_per_halfsweep(self._h, C.byref(v)))
        return v.value


class GraphDef:
    """Node count + edge list (src/graph.rs:4-79): `edges` is an (m, 2) int array.

    from_json / from_edge_csv read the reference's two graph formats with its
    error messages; bcc / fcc / diluted_cubic build the periodic crystal graphs
    its J-fitting runs on (N^3 cells; two, four and one node per cell)."""

    def __init__(self, n_nodes: int, edges):
        self.n_nodes = int(n_nodes)
        self.edges = np.asarray(edges, np.int64).reshape(-1, 2)

    @staticmethod
    def from_json(content: str) -> "GraphDef":
        """{"n_nodes": N, "edges": [[a, b], ...]} (graph.rs:44-79)."""
        import json

        root = json.loads(content)

        def u64(v):
            return isinstance(v, int) and not isinstance(v, bool) and v >= 0

        n = root.get("n_nodes") if isinstance(root, dict) else None
        if not u64(n):
            raise ValueError("missing n_nodes")
        ev = root.get("edges")
        if not isinstance(ev, list):
            raise ValueError("missing edges")
        edges = []
        for e in ev:
            if not isinstance(e, list):
                raise ValueError("edge entry is not a 2-element array")
            if len(e) != 2:
                raise ValueError("edge entry must have exactly 2 indices")
            if not (u64(e[0]) and u64(e[1])):
                raise ValueError("edge index is not an integer")
            edges.append((e[0], e[1]))
        return GraphDef(n, np.array(edges, np.int64).reshape(-1, 2))

    @staticmethod
    def from_edge_csv(content: str) -> "GraphDef":
        """Lines "i,j" ('#' comments and blank lines skipped); n_nodes = max
        index + 1 (graph.rs:11-41)."""
        edges, top = [], 0
        for line in content.splitlines():
            t = line.strip()
            if not t or t.startswith("#"):
                continue
            parts = t.split(",")
            if len(parts) < 2:
                raise ValueError(f"bad edge line: {t}")
            i, j = int(parts[0].strip()), int(parts[1].strip())
            if i < 0 or j < 0:
                raise ValueError(f"bad edge line: {t}")
            top = max(top, i, j)
            edges.append((i, j))
        return GraphDef(top + 1, np.array(edges, np.int64).reshape(-1, 2))

    def to_json(self) -> str:
        pairs = ", ".join(f"[{int(a)}, {int(b)}]" for a, b in self.edges)
        return f'{{"n_nodes": {self.n_nodes}, "edges": [{pairs}]}}'

    def degrees(self) -> np.ndarray:
        d = np.zeros(self.n_nodes, np.int64)
        np.add.at(d, self.edges[:, 0], 1)
        np.add.at(d, self.edges[:, 1], 1)
        return d

    @staticmethod
    def bcc(n: int) -> "GraphDef":
        """Body-centred cubic, n^3 cells (n >= 2): corner node (x,y,z) is
        (x n + y) n + z, the centre of cell (x,y,z) is n^3 + that; each centre
        bonds to the 8 corners of its cell (coordination 8, 4 n^3 bonds)."""
        if n < 2:
            raise ValueError("bcc needs n >= 2")
        x, y, z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        cell = ((x * n + y) * n + z).reshape(-1)
        out = []
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    corner = ((((x + dx) % n) * n + (y + dy) % n) * n + (z + dz) % n).reshape(-1)
                    out.append(np.stack([corner, n ** 3 + cell], 1))
        return GraphDef(2 * n ** 3, np.concatenate(out))

    @staticmethod
    def fcc(n: int) -> "GraphDef":
        """Face-centred cubic, n^3 cells (n >= 2): the points (a,b,c) of a 2n
        periodic grid with a+b+c even, numbered in (a,b,c) order, each bonded to
        the 12 points at (+-1,+-1,0) and its permutations (12 n^3 bonds)."""
        if n < 2:
            raise ValueError("fcc needs n >= 2")
        m = 2 * n
        a, b, c = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
        keep = ((a + b + c) % 2 == 0).reshape(-1)
        index = np.full(m ** 3, -1, np.int64)
        index[keep] = np.arange(int(keep.sum()))
        pa, pb, pc = a.reshape(-1)[keep], b.reshape(-1)[keep], c.reshape(-1)[keep]
        me = index[((pa * m + pb) * m + pc)]
        out = []
        for da, db, dc in ((1, 1, 0), (1, -1, 0), (1, 0, 1), (1, 0, -1), (0, 1, 1), (0, 1, -1)):
            nb = index[((((pa + da) % m) * m + (pb + db) % m) * m + (pc + dc) % m)]
            out.append(np.stack([me, nb], 1))
        return GraphDef(4 * n ** 3, np.concatenate(out))

    @staticmethod
    def diluted_cubic(n: int, p_remove: float, seed: int = 0) -> "GraphDef":
        """Periodic simple cubic n^3 (n >= 3) with round(p_remove * 3 n^3) of its
        3 n^3 bonds removed, chosen by a permutation from numpy's PCG64 stream
        of `seed`; the kept bonds stay in lattice order."""
        if n < 3:
            raise ValueError("diluted_cubic needs n >= 3")
        x, y, z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        me = ((x * n + y) * n + z).reshape(-1)
        out = [np.stack([me, ((((x + 1) % n) * n + y) * n + z).reshape(-1)], 1),
               np.stack([me, ((x * n + (y + 1) % n) * n + z).reshape(-1)], 1),
               np.stack([me, ((x * n + y) * n + (z + 1) % n).reshape(-1)], 1)]
        e = np.concatenate(out)
        if not 0.0 <= p_remove <= 1.0:
            raise ValueError("p_remove must be in [0, 1]")
        drop = int(round(p_remove * len(e)))
        keep = np.ones(len(e), bool)
        keep[np.random.default_rng(seed).permutation(len(e))[:drop]] = False
        return GraphDef(n ** 3, e[keep])


class GraphBatch:
    """`replicas` Ising replicas of one graph (node count + edge list, GraphDef of
    src/graph.rs:4-79) with device replica exchange: the GB300 form of
    run_ising_jfit (src/bin/gpu_jfit.rs:172-297).

    Sites are updated colour class by colour class of a greedy proper colouring
    in node order (num_colours()); at most 65536 nodes, degree 12 and 1024
    replicas; self-loops are rejected."""

    def __init__(self, n_nodes: int, edges, replicas: int, seed: int = 42):
        e = np.ascontiguousarray(edges, np.int32).reshape(-1)
        self.n, self.replicas = int(n_nodes), int(replicas)
        h = C.c_void_p()
        _check(lib().isg_graph_create(C.byref(h), self.n, _ptr(e) if len(e) else None,
                                      len(e) // 2, self.replicas, int(seed)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().isg_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_colours(self) -> int:
        v = C.c_int()
        _check(lib().isg_graph_num_colours(self._h, C.byref(v)))
        return v.value

    def set_temperatures(self, temps, J: float = 1.0) -> None:
        t = np.ascontiguousarray(temps, np.float64)
        if len(t) != self.replicas:
            raise IsingError(-1, "need one temperature per replica slot")
        _check(lib().isg_graph_set_temperatures(self._h, _ptr(t), float(J)))

    def step(self, n_sweeps: int = 1) -> None:
        _check(lib().isg_graph_step(self._h, int(n_sweeps)))

    def reset_sampling(self) -> None:
        _check(lib().isg_graph_reset_sampling(self._h))

    def pt_run(self, n_sweeps: int, exchange_every: int, measure_every: int = 1):
        """(slot, bond, mag) records of shape (rows, replicas)."""
        rows = n_sweeps // measure_every + 1
        t = np.zeros((rows, self.replicas), np.int32)
        b = np.zeros((rows, self.replicas), np.int64)
        m = np.zeros((rows, self.replicas), np.int64)
        n = C.c_int64()
        _check(lib().isg_graph_pt_run(self._h, int(n_sweeps), int(exchange_every),
                                      int(measure_every), _ptr(t), _ptr(b), _ptr(m), rows,
                                      C.byref(n)))
        return t[:n.value], b[:n.value], m[:n.value]

    def accepted(self) -> int:
        v = C.c_int64()
        _check(lib().isg_graph_get_accepted(self._h, C.byref(v)))
        return v.value

    def get_spins(self, r: int) -> np.ndarray:
        out = np.zeros(self.n, np.int8)
        _check(lib().isg_graph_get_spins(self._h, int(r), _ptr(out)))
        return out

    def r2t(self) -> np.ndarray:
        out = np.zeros(self.replicas, np.int32)
        _check(lib().isg_graph_get_r2t(self._h, _ptr(out)))
        return out


class ContinuousGraphBatch:
    """`replicas` continuous-spin replicas of one graph with device replica
    exchange: n_comp = 3 is run_heisenberg_jfit (cone Metropolis, half-angle
    `set_delta`, default 0.5; src/bin/gpu_jfit.rs:414-524), n_comp = 2 is
    run_xy_jfit (one single-cluster Wolff flip per sweep; gpu_jfit.rs:298-412).

    At most 16384 nodes, degree 64 and 1024 replicas; spins are FP32 unit
    vectors, energies and magnetisations FP64 sums."""

    def __init__(self, n_nodes: int, edges, replicas: int, n_comp: int, seed: int = 42):
        e = np.ascontiguousarray(edges, np.int32).reshape(-1)
        self.n, self.replicas, self.nc = int(n_nodes), int(replicas), int(n_comp)
        h = C.c_void_p()
        _check(lib().isg_cgraph_create(C.byref(h), self.n, _ptr(e) if len(e) else None,
                                       len(e) // 2, self.replicas, self.nc, int(seed)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().isg_cgraph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_colours(self) -> int:
        v = C.c_int()
        _check(lib().isg_cgraph_num_colours(self._h, C.byref(v)))
        return v.value

    def set_temperatures(self, temps, J: float = 1.0) -> None:
        t = np.ascontiguousarray(temps, np.float64)
        if len(t) != self.replicas:
            raise IsingError(-1, "need one temperature per replica slot")
        _check(lib().isg_cgraph_set_temperatures(self._h, _ptr(t), float(J)))

    def set_delta(self, delta: float) -> None:
        _check(lib().isg_cgraph_set_delta(self._h, float(delta)))

    def step(self, n_sweeps: int = 1) -> None:
        _check(lib().isg_cgraph_step(self._h, int(n_sweeps)))

    def reset_sampling(self) -> None:
        _check(lib().isg_cgraph_reset_sampling(self._h))

    def pt_run(self, n_sweeps: int, exchange_every: int, measure_every: int = 1):
        """(slot (rows, R), energy (rows, R), magnetisation (rows, R, n_comp))."""
        rows = n_sweeps // measure_every + 1
        t = np.zeros((rows, self.replicas), np.int32)
        e = np.zeros((rows, self.replicas), np.float64)
        m = np.zeros((rows, self.replicas, self.nc), np.float64)
        n = C.c_int64()
        _check(lib().isg_cgraph_pt_run(self._h, int(n_sweeps), int(exchange_every),
                                       int(measure_every), _ptr(t), _ptr(e), _ptr(m), rows,
                                       C.byref(n)))
        return t[:n.value], e[:n.value], m[:n.value]

    def accepted(self) -> int:
        v = C.c_int64()
        _check(lib().isg_cgraph_get_accepted(self._h, C.byref(v)))
        return v.value

    def moves(self) -> np.ndarray:
        out = np.zeros(self.replicas, np.int64)
        _check(lib().isg_cgraph_get_moves(self._h, _ptr(out)))
        return out

    def get_spins(self, r: int) -> np.ndarray:
        out = np.zeros((self.n, self.nc), np.float32)
        _check(lib().isg_cgraph_get_spins(self._h, int(r), _ptr(out)))
        return out

    def set_spins(self, r: int, spins) -> None:
        a = np.ascontiguousarray(spins, np.float32).reshape(self.n, self.nc)
        _check(lib().isg_cgraph_set_spins(self._h, int(r), _ptr(a)))

    def r2t(self) -> np.ndarray:
        out = np.zeros(self.replicas, np.int32)
        _check(lib().isg_cgraph_get_r2t(self._h, _ptr(out)))
        return out

    def sweep_count(self) -> int:
        v = C.c_uint64()
        _check(lib().isg_cgraph_get_sweep(self._h, C.byref(v)))
        return v.value


# ----------------------------------------------------------------- reweighting
# GPU forms of analysis/scripts/reweighting.py and of the reweighting steps of
# analysis/scripts/analyze_gpu_fss.py (names, arguments and results as there;
# the fine-grid tables are dicts of columns instead of DataFrames).

_MOM_SCALE = 2.0 ** -32


def _points(energy_lists):
    e = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64) for x in energy_lists]))
    nk = np.array([len(x) for x in energy_lists], np.float64)
    return e, np.ones(len(e)), nk


def _wham_call(e, c, mom, n_mom, beta, nk, beta_t, n_iter=100, tol=1e-8):
    bt = np.ascontiguousarray(beta_t, np.float64)
    out = np.zeros((len(bt), 3 + n_mom))
    f = np.zeros(len(beta))
    it = C.c_int()
    b = np.ascontiguousarray(beta, np.float64)
    mom_p = _ptr(mom) if n_mom else None
    _check(lib().isg_wham(_ptr(e), _ptr(c), mom_p, n_mom, len(e), _ptr(b),
                          _ptr(np.ascontiguousarray(nk, np.float64)), len(b), int(n_iter),
                          float(tol), _ptr(bt), len(bt), _ptr(out), _ptr(f), C.byref(it)))
    return out, f, it.value


def single_histogram(energies, beta_sim, beta_target):
    """reweighting.py:15-37: normalised weights exp(-(beta_target - beta_sim) E)."""
    e = np.ascontiguousarray(energies, np.float64)
    w = np.zeros(len(e))
    b = np.array([float(beta_sim)])
    _check(lib().isg_wham_weights(_ptr(e), _ptr(np.ones(len(e))), len(e), _ptr(b),
                                  _ptr(np.array([float(len(e))])), 1, 1, 1e-8,
                                  float(beta_target), _ptr(w), None, None))
    return w


def reweight_observable(observable, weights):
    """reweighting.py:40-42."""
    return np.sum(observable * weights)


def wham_reweight(energy_lists, beta_list, beta_target, n_iter=100, tol=1e-8):
    """reweighting.py:45-105: (normalised weights of all samples, simulation index)."""
    e, c, nk = _points(energy_lists)
    b = np.ascontiguousarray(beta_list, np.float64)
    w = np.zeros(len(e))
    _check(lib().isg_wham_weights(_ptr(e), _ptr(c), len(e), _ptr(b), _ptr(nk), len(b),
                                  int(n_iter), float(tol), float(beta_target), _ptr(w), None,
                                  None))
    sim = np.concatenate([np.full(len(x), k) for k, x in enumerate(energy_lists)])
    return w, sim


def reweight_binder(energy_lists, mag_lists, beta_list, beta_targets):
    """reweighting.py:108-143: (T, U) at the target betas (one WHAM solve)."""
    e, c, nk = _points(energy_lists)
    m = np.concatenate([np.asarray(x, np.float64) for x in mag_lists])
    mom = np.ascontiguousarray(np.stack([m * m, (m * m) * (m * m)], axis=1))
    bt = np.asarray(beta_targets, np.float64)
    out, _, _ = _wham_call(e, c, mom, 2, beta_list, nk, bt)
    m2, m4 = out[:, 3], out[:, 4]
    U = np.where(m2 > 0, 1.0 - m4 / (3.0 * np.where(m2 > 0, m2, 1.0) ** 2), 0.0)
    return 1.0 / bt, U


def _fine_table(T_fine, beta_list, V, avg, e_lists, m_lists):
    """Columns of analyze_gpu_fss.py's fine-grid tables from averages avg[t] =
    (logZ, <E>, <E^2>, <m>, <m^2>, <m^4>) and the leave-one-block-out
    single-histogram jackknife (20 blocks) of the closest simulation."""
    b = np.asarray(beta_list, np.float64)
    T = np.asarray(T_fine, np.float64)
    bt = 1.0 / T
    kb = np.array([int(np.argmin(np.abs(1.0 / b - t))) for t in T])
    offs = np.concatenate([[0], np.cumsum([len(x) for x in e_lists])])
    e, c, _ = _points(e_lists)
    m = np.concatenate([np.asarray(x, np.float64) for x in m_lists])
    mom = np.ascontiguousarray(np.stack([m, m * m, (m * m) * (m * m)], axis=1))
    nb = 20
    rows = len(T) * nb
    p0 = np.repeat(offs[kb], nb).astype(np.int64)
    bs = np.repeat(np.array([len(e_lists[k]) for k in kb]) // nb, nb).astype(np.int64)
    blk = np.tile(np.arange(nb, dtype=np.int64), len(T))
    p1 = p0 + nb * bs
    x0 = p0 + blk * bs
    x1 = x0 + bs
    jk = np.zeros((rows, 6))
    _check(lib().isg_reweight_single(_ptr(e), _ptr(c), _ptr(mom), 3, len(e), _ptr(p0), _ptr(p1),
                                     _ptr(x0), _ptr(x1),
                                     _ptr(np.ascontiguousarray(np.repeat(b[kb], nb))),
                                     _ptr(np.ascontiguousarray(np.repeat(bt, nb))), rows,
                                     _ptr(jk)))
    jk = jk.reshape(len(T), nb, 6)
    am, am2, am4 = avg[:, 3], avg[:, 4], avg[:, 5]
    ae, ae2 = avg[:, 1], avg[:, 2]
    chi = bt * V * (am2 - am ** 2)
    U = np.where(am2 > 1e-15, 1.0 - am4 / (3.0 * np.where(am2 > 1e-15, am2, 1.0) ** 2), 0.0)
    j1, j2, j4 = jk[:, :, 3], jk[:, :, 4], jk[:, :, 5]
    jc = bt[:, None] * V * (j2 - j1 ** 2)
    ju = np.where(j2 > 1e-15, 1.0 - j4 / (3.0 * np.where(j2 > 1e-15, j2, 1.0) ** 2), 0.0)
    f = (nb - 1.0) / nb
    return {"T": T, "M": am, "M2": am2, "M4": am4, "chi_conn": chi,
            "chi_err": np.sqrt(f * np.sum((jc - chi[:, None]) ** 2, axis=1)),
            "Cv": bt ** 2 * (ae2 - ae ** 2) / V, "U": U, "E": ae / V,
            "M_err": np.sqrt(f * np.sum((j1 - am[:, None]) ** 2, axis=1)),
            "U_err": np.sqrt(f * np.sum((ju - U[:, None]) ** 2, axis=1))}


def reweight_single_histogram(energy_lists, mag_lists, beta_list, T_fine, n: int):
    """analyze_gpu_fss.py:86-157: every T of the fine grid reweighted from the
    closest simulation (total energies, |m| per spin, V = n^3)."""
    b = np.asarray(beta_list, np.float64)
    T = np.asarray(T_fine, np.float64)
    kb = np.array([int(np.argmin(np.abs(1.0 / b - t))) for t in T])
    offs = np.concatenate([[0], np.cumsum([len(x) for x in energy_lists])])
    e, c, _ = _points(energy_lists)
    m = np.concatenate([np.asarray(x, np.float64) for x in mag_lists])
    mom = np.ascontiguousarray(np.stack([m, m * m, (m * m) * (m * m)], axis=1))
    avg = np.zeros((len(T), 6))
    p0 = np.ascontiguousarray(offs[kb], np.int64)
    p1 = np.ascontiguousarray(offs[kb + 1], np.int64)
    _check(lib().isg_reweight_single(_ptr(e), _ptr(c), _ptr(mom), 3, len(e), _ptr(p0), _ptr(p1),
                                     None, None, _ptr(np.ascontiguousarray(b[kb])),
                                     _ptr(np.ascontiguousarray(1.0 / T)), len(T), _ptr(avg)))
    return _fine_table(T, b, float(n) ** 3, avg, energy_lists, mag_lists)


def wham_reweight_fine(energy_lists, mag_lists, beta_list, T_fine, n: int, n_iter=100,
                       tol=1e-8):
    """analyze_gpu_fss.py:160-243: WHAM over all simulations at every T of the
    fine grid; errors from the closest simulation's jackknife."""
    e, c, nk = _points(energy_lists)
    m = np.concatenate([np.asarray(x, np.float64) for x in mag_lists])
    mom = np.ascontiguousarray(np.stack([m, m * m, (m * m) * (m * m)], axis=1))
    T = np.asarray(T_fine, np.float64)
    avg, _, _ = _wham_call(e, c, mom, 3, beta_list, nk, 1.0 / T, n_iter, tol)
    return _fine_table(T, beta_list, float(n) ** 3, avg, energy_lists, mag_lists)


def wham_histograms(bonds, counters, temps, J: float, n_sites: float, T_fine, n_iter=100,
                    tol=1e-8):
    """WHAM over the exact energy histograms of one size (IsingBatch.histogram
    per slot: bonds[k], counters[k]): identical to WHAM over the samples, since
    every sample of a bin has the same energy E = -J B.  Returns columns T, E
    (per spin), Cv, M, M2, M4, U, chi_conn as analyze_gpu_fss.py defines them."""
    allb = np.unique(np.concatenate([np.asarray(x, np.int64) for x in bonds]))
    idx = {int(v): i for i, v in enumerate(allb)}
    P = len(allb)
    c = np.zeros(P)
    mom = np.zeros((P, 3))
    nk = np.zeros(len(temps))
    for k, (bk, ck) in enumerate(zip(bonds, counters)):
        pos = np.array([idx[int(v)] for v in bk], np.int64)
        ck = np.asarray(ck, np.uint64)
        np.add.at(c, pos, ck[:, 0].astype(np.float64))
        for j in range(3):
            np.add.at(mom[:, j], pos, ck[:, 1 + j].astype(np.float64) * _MOM_SCALE)
        nk[k] = float(ck[:, 0].sum())
    e = np.ascontiguousarray(-float(J) * allb.astype(np.float64))
    T = np.asarray(T_fine, np.float64)
    bt = 1.0 / T
    avg, f, it = _wham_call(e, np.ascontiguousarray(c), np.ascontiguousarray(mom), 3,
                            1.0 / np.asarray(temps, np.float64), nk, bt, n_iter, tol)
    V = float(n_sites)
    am, am2, am4 = avg[:, 3], avg[:, 4], avg[:, 5]
    return {"T": T, "E": avg[:, 1] / V, "Cv": bt ** 2 * (avg[:, 2] - avg[:, 1] ** 2) / V,
            "M": am, "M2": am2, "M4": am4,
            "U": np.where(am2 > 1e-15, 1.0 - am4 / (3.0 * np.where(am2 > 1e-15, am2, 1.0) ** 2),
                          0.0),
            "chi_conn": bt * V * (am2 - am ** 2), "f": f, "iterations": it}


# ----------------------------------------------------------------- binary files

TS_DTYPE = np.dtype([("temp_idx", "<u4"), ("replica", "<u4"), ("E", "<f8"), ("M", "<f8")])
MODELS = ("ising", "heisenberg", "xy")


def write_timeseries(path, model: str, n: int, temps, temp_idx, replica, E, M) -> None:
    """Binary timeseries through isg_ts_* (the layout include/isg.h documents)."""
    t = np.ascontiguousarray(temps, np.float64)
    h = C.c_void_p()
    _check(lib().isg_ts_open(C.byref(h), str(path).encode(), MODELS.index(model), int(n),
                             _ptr(t), len(t)))
    try:
        ti = np.ascontiguousarray(temp_idx, np.int32)
        rp = np.ascontiguousarray(replica, np.int32)
        ee = np.ascontiguousarray(E, np.float64)
        mm = np.ascontiguousarray(M, np.float64)
        _check(lib().isg_ts_append(h, _ptr(ti), _ptr(rp), _ptr(ee), _ptr(mm), len(ti)))
    finally:
        _check(lib().isg_ts_close(h))


def read_timeseries(path) -> dict:
    """A binary timeseries: {model, n, temps, records (TS_DTYPE array)}."""
    raw = Path(path).read_bytes()
    if raw[:8] != b"ISGTSER1":
        raise ValueError(f"{path}: not an ISGTSER1 timeseries")
    hb, model, n, nt = np.frombuffer(raw, "<u4", 4, 8)
    temps = np.frombuffer(raw, "<f8", int(nt), 32)
    rec = np.frombuffer(raw, TS_DTYPE, offset=int(hb))
    return {"model": MODELS[int(model)], "n": int(n), "temps": temps.copy(), "records": rec}


def timeseries_lists(ts: dict):
    """(energy_lists, mag_lists, beta_list) of a timeseries as
    analyze_gpu_fss.py:60-83 builds them: total energies E V and |m|, per
    temperature index in order."""
    V = float(ts["n"]) ** 3
    rec = ts["records"]
    el, ml, bl = [], [], []
    for t, T in enumerate(ts["temps"]):
        sel = rec["temp_idx"] == t
        if not sel.any():
            continue
        el.append(rec["E"][sel] * V)
        ml.append(rec["M"][sel].copy())
        bl.append(1.0 / T)
    return el, ml, np.array(bl)


def read_histograms(path) -> dict:
    """A histogram file: {dim, n, J, temps, bonds[t], counters[t] (n, 4)}."""
    raw = Path(path).read_bytes()
    if raw[:8] != b"ISGHIST1":
        raise ValueError(f"{path}: not an ISGHIST1 histogram file")
    hb, dim, n, nt = np.frombuffer(raw, "<u4", 4, 8)
    J = float(np.frombuffer(raw, "<f8", 1, 24)[0])
    temps = np.frombuffer(raw, "<f8", int(nt), 32).copy()
    off = int(hb)
    bonds, cnt = [], []
    for _ in range(int(nt)):
        lo, nbins = np.frombuffer(raw, "<i8", 2, off)
        off += 16
        c = np.frombuffer(raw, "<u8", 4 * int(nbins), off).reshape(-1, 4).copy()
        off += 32 * int(nbins)
        bonds.append(int(lo) + 4 * np.arange(int(nbins), dtype=np.int64))
        cnt.append(c)
    return {"dim": int(dim), "n": int(n), "J": J, "temps": temps, "bonds": bonds,
            "counters": cnt}


class LatticeGpu:
    """Mirror of LatticeGpu (src/cuda/lattice_gpu.rs:9-189): one cubic replica.

    `step(beta, j, h)` sweeps once (colour 0 then colour 1); `measure_gpu(j)`
    returns (E/N^3, |M|/N^3) synchronously; `energy_gpu(j)` the total energy.
    Spins start hot from the seeded Philox stream (the reference's are
    unseeded, lattice_gpu.rs:38-40)."""

    def __init__(self, n: int, seed: int):
        self.n = int(n)
        self._b = IsingBatch([self.n], 1, seed=seed, dim=3)
        self._key = None

    def _set(self, beta: float, j: float, h: float) -> None:
        key = (float(beta), float(j), float(h))
        if key != self._key:
            self._b.set_temperatures([1.0 / key[0]], J=key[1], h=key[2])
            self._key = key

    def step(self, beta: float, j: float, h: float) -> None:
        self._set(beta, j, h)
        self._b.step(1)

    def warm_up(self, beta: float, j: float, h: float, sweeps: int) -> None:
        self._set(beta, j, h)
        self._b.step(sweeps)

    def measure_gpu(self, j: float) -> tuple[float, float]:
        # The reference reduction sums -J s_i s_j only (reduce_kernel.cu:52-56):
        # the field term is not part of the measured energy.
        b, m = self._b.measure()
        n3 = float(self.n) ** 3
        return -float(j) * float(b[0]) / n3, abs(float(m[0])) / n3

    def energy_gpu(self, j: float) -> float:
        b, _ = self._b.measure()
        return -float(j) * float(b[0])

    def get_spins(self) -> np.ndarray:
        return self._b.get_spins(0, 0)

    def measure(self, temperature: float, j: float, h: float, samples: int) -> Observables:
        """src/cuda/lattice_gpu.rs:190-251: `samples` sweeps at `temperature`, each
        followed by a measurement of E (with the field term) and M; chi from the
        signed magnetisation.  E and M come from the sweep's fused integer sums
        instead of a spin copy per sample."""
        if samples < 1:
            raise IsingError(-1, "samples must be at least 1")
        T = float(temperature)
        if self._key != ("T", T, float(j), float(h)):
            self._b.set_temperatures([T], J=float(j), h=float(h))
            self._key = ("T", T, float(j), float(h))
        b, m = self._b.run_schedule(None, int(samples), 1, 0)
        return _observables(T, b[:, 0], m[:, 0], float(j), float(h), float(self.n) ** 3)

    def domain_wall_density(self) -> float:
        """src/cuda/lattice_gpu.rs:253-281: fraction of the 3 N^3 forward bonds whose
        spins differ, from the device bond sum B = (equal - unequal):
        walls = (3 N^3 - B) / 2."""
        b, _ = self._b.measure()
        bonds = 3 * self.n ** 3
        walls = (bonds - int(b[0])) // 2
        return walls / bonds


class ContinuousBatch:
    """Every (size, replica) O(n) lattice (n_comp 2 = XY, 3 = Heisenberg)."""

    def __init__(self, sizes, replicas: int, n_comp: int, seed: int = 42):
        self.sizes = [int(s) for s in sizes]
        self.replicas = int(replicas)
        self.n_comp = int(n_comp)
        self.seed = int(seed)
        arr = np.ascontiguousarray(self.sizes, np.int32)
        h = C.c_void_p()
        _check(lib().isg_cont_create(C.byref(h), _ptr(arr), len(self.sizes), self.replicas,
                                     self.n_comp, self.seed))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().isg_cont_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_total(self) -> int:
        return len(self.sizes) * self.replicas

    def nsites(self, s: int) -> int:
        return self.sizes[s] ** 3

    def set_stream(self, stream) -> None:
        h = _stream_handle(stream)
        _check(lib().isg_cont_set_stream(self._h, C.c_void_p(h) if h else None))

    def set_temperatures(self, temps, J: float = 1.0) -> None:
        t = np.asarray(temps, np.float64)
        if t.ndim == 1 and len(t) == self.replicas:
            t = np.tile(t, len(self.sizes))
        t = np.ascontiguousarray(t.reshape(-1), np.float64)
        _check(lib().isg_cont_set_temperatures(self._h, _ptr(t), float(J)))
        self.temps = t.reshape(len(self.sizes), self.replicas)
        self.J = float(J)

    def sweep(self, n_sweeps: int = 1, delta: float = 0.5, n_overrelax: int = 5) -> None:
        _check(lib().isg_cont_sweep(self._h, int(n_sweeps), float(delta), int(n_overrelax)))

    def overrelax(self, colour: int) -> None:
        _check(lib().isg_cont_overrelax(self._h, int(colour)))

    def metropolis(self, colour: int, delta: float) -> None:
        _check(lib().isg_cont_metropolis(self._h, int(colour), float(delta)))

    def normalize(self) -> None:
        _check(lib().isg_cont_normalize(self._h))

    def measure(self):
        """Returns (E [n_total], M [n_total, 3], bond sums [n_total, 6]):
        bond sums = sum_i S_i.S_{i+a} (a = x,y,z) then sum_i (S_i x S_{i+a})_z."""
        e = np.zeros(self.n_total, np.float64)
        m = np.zeros((self.n_total, 3), np.float64)
        hb = np.zeros((self.n_total, 6), np.float64)
        _check(lib().isg_cont_measure(self._h, _ptr(e), _ptr(m), _ptr(hb)))
        return e, m, hb

    def exchange(self, parity: int = -1) -> np.ndarray:
        acc = np.zeros(len(self.sizes), np.int64)
        _check(lib().isg_cont_exchange(self._h, int(parity), _ptr(acc)))
        return acc

    def reset_sampling(self) -> None:
        _check(lib().isg_cont_reset_sampling(self._h))

    def pt_run(self, n_sweeps: int, exchange_every: int, measure_every: int, delta: float = 0.5,
               n_overrelax: int = 5, renorm_every: int = 100):
        """Returns (slot, E, M[...,3], bond sums[...,6]) per record."""
        rows = n_sweeps // measure_every + 1
        nt = self.n_total
        t = np.zeros((rows, nt), np.int32)
        e = np.zeros((rows, nt), np.float64)
        m = np.zeros((rows, nt, 3), np.float64)
        hb = np.zeros((rows, nt, 6), np.float64)
        n = C.c_int64()
        _check(lib().isg_cont_pt_run(self._h, int(n_sweeps), int(exchange_every),
                                     int(measure_every), float(delta), int(n_overrelax),
                                     int(renorm_every), _ptr(t), _ptr(e), _ptr(m), _ptr(hb), rows,
                                     C.byref(n)))
        k = n.value
        return t[:k], e[:k], m[:k], hb[:k]

    def r2t(self) -> np.ndarray:
        out = np.zeros(self.n_total, np.int32)
        _check(lib().isg_cont_get_r2t(self._h, _ptr(out)))
        return out

    def get_spins(self, s: int, r: int) -> np.ndarray:
        out = np.zeros(self.nsites(s) * self.n_comp, np.float32)
        _check(lib().isg_cont_get_spins(self._h, s, r, _ptr(out)))
        return out.reshape(-1, self.n_comp)

    def set_spins(self, s: int, r: int, spins) -> None:
        a = np.ascontiguousarray(spins, np.float32).reshape(-1)
        _check(lib().isg_cont_set_spins(self._h, s, r, _ptr(a)))

    def accepted(self) -> np.ndarray:
        out = np.zeros(len(self.sizes), np.int64)
        _check(lib().isg_cont_get_accepted(self._h, _ptr(out)))
        return out

    def metropolis_accepted(self) -> np.ndarray:
        out = np.zeros(self.n_total, np.int64)
        _check(lib().isg_cont_get_metro_accepted(self._h, _ptr(out)))
        return out

    def sync(self) -> None:
        _check(lib().isg_cont_sync(self._h))

    def set_fused_measure(self, enable: bool = True) -> None:
        """Measured PT sweeps: measurement fused into the last half-sweep (same bits)."""
        _check(lib().isg_cont_set_fused_measure(self._h, int(bool(enable))))

    def time_kernels(self, n: int = 10) -> np.ndarray:
        """Mean ms of an overrelaxation half-sweep, a Metropolis half-sweep, a
        measurement and a fused Metropolis + measurement half-sweep."""
        out = np.zeros(4, np.float32)
        _check(lib().isg_cont_time_kernels(self._h, int(n), _ptr(out)))
        return out

    def sites_per_sweep(self) -> int:
        v = C.c_int64()
        _check(lib().isg_cont_sites_per_sweep(self._h, C.byref(v)))
        return v.value


def tune_delta(batch: "ContinuousBatch", delta: float = 0.5, n_overrelax: int = 4,
               target: float = 0.5, rounds: int = 12, sweeps: int = 20) -> float:
    """Adjust the Metropolis cone half-angle so that about `target` of the
    proposals are accepted (averaged over all replicas): delta is scaled by
    acc/target (clamped to [1/2, 2] per round) after each burst of sweeps.
    Returns the tuned delta; the sweeps advance the chains (use during warm-up)."""
    d = float(delta)
    sites = batch.sites_per_sweep()
    for _ in range(rounds):
        a0 = batch.metropolis_accepted().sum()
        batch.sweep(sweeps, d, n_overrelax)
        acc = (batch.metropolis_accepted().sum() - a0) / (sites * sweeps)
        d = min(math.pi, d * min(2.0, max(0.5, acc / target)))
    return d


class ContinuousGpuLattice:
    """Mirror of ContinuousGpuLattice (src/cuda/gpu_lattice_continuous.rs:9-245).

    `sweep(beta, j, delta, n_overrelax)` runs n_overrelax overrelaxation sweeps
    then one Metropolis sweep (the reference GPU order, :112-173);
    `measure_gpu(j)` returns (E_total, mx, my, mz)."""

    def __init__(self, n: int, n_comp: int, seed: int):
        self.n, self.n_comp = int(n), int(n_comp)
        self._b = ContinuousBatch([self.n], 1, self.n_comp, seed=seed)
        self._key = None

    def sweep(self, beta: float, j: float, delta: float, n_overrelax: int) -> None:
        key = (float(beta), float(j))
        if key != self._key:
            self._b.set_temperatures([1.0 / key[0]], J=key[1])
            self._key = key
        self._b.sweep(1, delta, n_overrelax)

    def measure_gpu(self, j: float):
        e, m, _ = self._b.measure()
        scale = float(j) / (self._key[1] if self._key else 1.0)
        return float(e[0]) * scale, float(m[0, 0]), float(m[0, 1]), float(m[0, 2])

    def measure_raw(self):
        return self.measure_gpu(1.0)
