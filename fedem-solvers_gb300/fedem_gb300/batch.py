"""Batched GPU execution of many FEDEM models (the ``fgpu_*`` C ABI).

``Model`` holds the host-side set-up of one model (parse, element matrices,
numbering, multifrontal symbolic analysis); ``Batch`` uploads models to HBM
and advances all of them to their end time together, one Newton iteration
per model per batched iteration.
"""
import ctypes
import os

import numpy as np

from . import FedemException, _argv, load_library

_P = ctypes.POINTER


def _ptr(a, ctype):
    return a.ctypes.data_as(_P(ctype))


class Model:
    """Host set-up of one model from solver-input text and solver options."""

    def __init__(self, fsi, options=(), lib=None):
        self._lib = lib or load_library()
        argc, argv = _argv(["fedem_solver"] + list(options))
        h = ctypes.c_void_p()
        rc = self._lib.fgpu_model_create(fsi.encode() if isinstance(fsi, str) else fsi, argc, argv, ctypes.byref(h))
        if rc != 0:
            raise FedemException(f"model set-up failed ({rc}): " + self._lib.fgpu_last_error().decode())
        self._h = h
        s = np.zeros(8, dtype=np.int64)
        self._lib.fgpu_model_sizes(self._h, _ptr(s, ctypes.c_longlong))
        (self.ntri, self.ndof, self.neq, self.nel, self.nnz, self.nfront, self.max_front,
         self.levels) = (int(v) for v in s)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fgpu_model_destroy(self._h)
            self._h = None

    __del__ = close

    def meqn(self):
        v = np.zeros(self.ndof, dtype=np.int32)
        self._lib.fgpu_model_meqn(self._h, _ptr(v, ctypes.c_int))
        return v

    def csr_pattern(self):
        rp = np.zeros(self.neq + 1, dtype=np.int32)
        ci = np.zeros(self.nnz, dtype=np.int32)
        self._lib.fgpu_model_csr_pattern(self._h, _ptr(rp, ctypes.c_int), _ptr(ci, ctypes.c_int))
        return rp, ci

    def symbolic(self):
        perm = np.zeros(self.neq, dtype=np.int32)
        info = np.zeros((self.nfront, 4), dtype=np.int32)
        self._lib.fgpu_model_symbolic(self._h, _ptr(perm, ctypes.c_int), _ptr(info, ctypes.c_int))
        return perm, info

    def element_matrix(self, iel, which):
        m = np.zeros(144)
        rc = self._lib.fgpu_model_element_matrix(self._h, iel, which, _ptr(m, ctypes.c_double))
        if rc != 0:
            raise FedemException("element_matrix: bad argument")
        return m.reshape((12, 12), order="F")


def create_models(cases, threads=None, lib=None):
    """Model set-up (fgpu_model_create) of many (fsi, options, ...) cases on the
    host's threads; the C call releases the interpreter lock and keeps no
    shared state, so the models are built in parallel.  Returns them in order."""
    from concurrent.futures import ThreadPoolExecutor

    lib = lib or load_library()
    cases = list(cases)
    n = threads or os.cpu_count() or 1
    # largest models first for the balance, results back in input order
    order = sorted(range(len(cases)), key=lambda k: -len(cases[k][0]))
    out = [None] * len(cases)

    def one(k):
        out[k] = Model(cases[k][0], cases[k][1], lib=lib)

    with ThreadPoolExecutor(max_workers=max(1, n)) as ex:
        list(ex.map(one, order))
    return out


def set_device(ordinal, lib=None):
    """Selects the CUDA device of every batch/server created afterwards
    (fgpu_set_device); returns (ordinal, PCI bus id)."""
    lib = lib or load_library()
    if lib.fgpu_set_device(int(ordinal)) != 0:
        raise FedemException("fgpu_set_device failed: " + lib.fgpu_last_error().decode())
    return get_device(lib)


def get_device(lib=None):
    lib = lib or load_library()
    dev = ctypes.c_int(-1)
    bus = ctypes.create_string_buffer(64)
    if lib.fgpu_get_device(ctypes.byref(dev), bus, 64) != 0:
        raise FedemException("fgpu_get_device failed: " + lib.fgpu_last_error().decode())
    return dev.value, bus.value.decode()


def measure_fp64_peak(lib=None):
    """Measured FP64 FMA rate of the current device: (TFLOP/s, ms of the best
    launch) from fgpu_measure_fp64_peak."""
    lib = lib or load_library()
    tf, ms = ctypes.c_double(0.0), ctypes.c_double(0.0)
    if lib.fgpu_measure_fp64_peak(ctypes.byref(tf), ctypes.byref(ms)) != 0:
        raise FedemException("fgpu_measure_fp64_peak failed")
    return tf.value, ms.value


def measure_tf32_mma_peak(lib=None):
    """Measured TF32 rate of mma.sync m16n8k8 (FP32 accumulation) on the current
    device: (TFLOP/s, ms of the best launch) from fgpu_measure_tf32_mma_peak."""
    lib = lib or load_library()
    tf, ms = ctypes.c_double(0.0), ctypes.c_double(0.0)
    if lib.fgpu_measure_tf32_mma_peak(ctypes.byref(tf), ctypes.byref(ms)) != 0:
        raise FedemException("fgpu_measure_tf32_mma_peak failed")
    return tf.value, ms.value


class Batch:
    """Models resident on the GPU, advanced together (mixed or FP64)."""

    def __init__(self, models, mixed=False, sweeps=0, lib=None):
        self._lib = lib or load_library()
        self.models = list(models)
        arr = (ctypes.c_void_p * len(self.models))(*[m._h for m in self.models])
        h = ctypes.c_void_p()
        rc = self._lib.fgpu_batch_create(len(self.models), arr, 1 if mixed else 0, int(sweeps), ctypes.byref(h))
        if rc != 0:
            raise FedemException(f"batch create failed ({rc}): " + self._lib.fgpu_last_error().decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fgpu_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def run(self, max_batched=0):
        """Runs every model to its end time; returns the run statistics."""
        s = np.zeros(10, dtype=np.int64)
        rc = self._lib.fgpu_batch_run(self._h, int(max_batched), _ptr(s, ctypes.c_longlong))
        if rc != 0:
            raise FedemException(f"batch run failed ({rc}): " + self._lib.fgpu_last_error().decode())
        keys = ("newton_iterations", "time_steps", "batched_iterations", "models_done", "models_failed",
                "kernels_per_iteration", "wall_us", "device_us", "h2d_bytes")
        return {k: int(v) for k, v in zip(keys, s)}

    def step(self, model):
        st = ctypes.c_int()
        rc = self._lib.fgpu_batch_step(self._h, model, ctypes.byref(st))
        if rc != 0:
            raise FedemException("step failed: " + self._lib.fgpu_last_error().decode())
        return st.value

    def info(self, model):
        st, ss, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        steps, its = ctypes.c_longlong(), ctypes.c_longlong()
        self._lib.fgpu_batch_model_info(self._h, model, ctypes.byref(st), ctypes.byref(ss), ctypes.byref(t),
                                        ctypes.byref(steps), ctypes.byref(its))
        return {"state": st.value, "status": ss.value, "time": t.value, "steps": steps.value,
                "iterations": its.value}

    def triads(self, model):
        ur = np.zeros(12 * self.models[model].ntri)
        self._lib.fgpu_batch_get_triads(self._h, model, _ptr(ur, ctypes.c_double))
        return ur.reshape((-1, 4, 3)).transpose(0, 2, 1)  # (ntri, 3, 4)

    def all_triads(self, out=None):
        n = 12 * sum(m.ntri for m in self.models)
        if out is None:
            out = np.zeros(n)
        self._lib.fgpu_batch_get_all_triads(self._h, _ptr(out, ctypes.c_double))
        return out

    def newton_values(self, model):
        v = np.zeros(self.models[model].nnz)
        self._lib.fgpu_batch_get_newton_values(self._h, model, _ptr(v, ctypes.c_double))
        return v

    def vector(self, model, which):
        v = np.zeros(self.models[model].neq)
        self._lib.fgpu_batch_get_vector(self._h, model, which, _ptr(v, ctypes.c_double))
        return v

    def snapshot(self):
        if self._lib.fgpu_batch_snapshot(self._h) != 0:
            raise FedemException("snapshot failed: " + self._lib.fgpu_last_error().decode())

    def restore(self):
        if self._lib.fgpu_batch_restore(self._h) != 0:
            raise FedemException("restore failed: " + self._lib.fgpu_last_error().decode())

    def phase_timings(self, reset=False):
        """(samples, [element ms, factor + first forward ms, other solve ms, second forward ms,
        back substitution ms], active elements) sampled inside run().  The back
        substitution is the one launched on its own: the first solve's, or the
        second solve's where the first runs inside the factorisation's launch
        (batches without large fronts)."""
        ms = np.zeros(5)
        el = ctypes.c_longlong()
        n = self._lib.fgpu_batch_phase_timings_n(self._h, _ptr(ms, ctypes.c_double), 5, ctypes.byref(el),
                                                 1 if reset else 0)
        return int(n), ms, int(el.value)

    def device(self):
        """CUDA device ordinal the batch was uploaded to."""
        return int(self._lib.fgpu_batch_device(self._h))

    def time_factor(self, reps=10):
        """(ms per launch, algorithmic bytes per launch) of the factorisation fused
        with the first forward elimination, every model factoring."""
        out = np.zeros(2)
        if self._lib.fgpu_batch_time_factor(self._h, int(reps), _ptr(out, ctypes.c_double)) != 0:
            raise FedemException("time_factor failed: " + self._lib.fgpu_last_error().decode())
        return float(out[0]), float(out[1])

    def set_launch_shape(self, panel, forward_warps, backward_warps, large_cluster):
        """Fixes the multifrontal launch shapes (before the first run) instead of
        the autotuner's probe: panel 0 (shuffles), 1 (register-blocked, blocks of
        8) or 2 (blocks of 4, fronts up to 32 rows); warps 4, 8 or 16; cluster
        2, 4, 8 or 16.  No shape changes a result bit."""
        sh = (ctypes.c_int * 4)(panel, forward_warps, backward_warps, large_cluster)
        if self._lib.fgpu_batch_set_launch_shape(self._h, sh) != 0:
            raise FedemException("set_launch_shape failed: " + self._lib.fgpu_last_error().decode())

    def launch_shape(self):
        """({panel, forward_warps, backward_warps, large_cluster}, probe ms, tuned)."""
        sh = (ctypes.c_int * 4)()
        ms = ctypes.c_double(0.0)
        tuned = self._lib.fgpu_batch_launch_shape(self._h, sh, ctypes.byref(ms))
        keys = ("panel", "forward_warps", "backward_warps", "large_cluster")
        return dict(zip(keys, list(sh))), ms.value, tuned == 1

    def assemble_newton(self, model, sM, sC, sK):
        """N = sM M + sC C + sK K of the model's current state, assembled on the
        GPU (read it with newton_values); between the model's steps."""
        if self._lib.fgpu_batch_assemble_newton(self._h, model, sM, sC, sK) != 0:
            raise FedemException("assemble_newton failed: " + self._lib.fgpu_last_error().decode())

    def factor(self, model):
        """LDL^T of the assembled N: the number of negative pivots; raises on a
        singular pivot (code -3) or an error."""
        rc = self._lib.fgpu_batch_factor(self._h, model)
        if rc < 0:
            raise FedemException(f"factor failed ({rc}): " + self._lib.fgpu_last_error().decode())
        return rc

    def solve(self, model, rhs):
        """Solutions of N x = b for b = rhs (neq values, or nrhs x neq)."""
        b = np.ascontiguousarray(np.array(rhs, dtype=np.float64))
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        if self._lib.fgpu_batch_solve(self._h, model, _ptr(b, ctypes.c_double), nrhs) != 0:
            raise FedemException("solve failed: " + self._lib.fgpu_last_error().decode())
        return b

    def results_open(self, directory, double=True):
        """Starts the results database: one file per model, <directory>/model<k>.res,
        a record of the current state now and one per completed time step
        (read it with fedem_gb300.results.read_results)."""
        if self._lib.fgpu_batch_results_open(self._h, str(directory).encode(), 1 if double else 0) != 0:
            raise FedemException("results_open failed: " + self._lib.fgpu_last_error().decode())

    def results_close(self):
        if self._lib.fgpu_batch_results_close(self._h) != 0:
            raise FedemException("results_close failed: " + self._lib.fgpu_last_error().decode())

    def norms(self, model):
        v = np.zeros(18)
        self._lib.fgpu_batch_get_norms(self._h, model, _ptr(v, ctypes.c_double))
        return v


class Server:
    """Continuous batching of simulation requests (fgpu_server_* C ABI)."""

    def __init__(self, budget_bytes=64e9, mixed=True, sweeps=0, max_models_per_batch=0, min_batch=8,
                 max_wait=0.02, lib=None):
        self._lib = lib or load_library()
        h = ctypes.c_void_p()
        rc = self._lib.fgpu_server_create(float(budget_bytes), 1 if mixed else 0, int(sweeps),
                                          int(max_models_per_batch), int(min_batch), float(max_wait),
                                          ctypes.byref(h))
        if rc != 0:
            raise FedemException("server create failed: " + self._lib.fgpu_last_error().decode())
        self._h = h
        self._models = {}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fgpu_server_destroy(self._h)
            self._h = None

    __del__ = close

    def submit(self, model):
        rid = ctypes.c_int()
        if self._lib.fgpu_server_submit(self._h, model._h, ctypes.byref(rid)) != 0:
            raise FedemException("submit failed: " + self._lib.fgpu_last_error().decode())
        self._models[rid.value] = model  # keep the host model alive until done
        return rid.value

    def pump(self):
        n = self._lib.fgpu_server_pump(self._h)
        if n < 0:
            raise FedemException("pump failed: " + self._lib.fgpu_last_error().decode())
        return n

    def now(self):
        return self._lib.fgpu_server_now(self._h)

    def set_max_engines(self, n):
        """At most n engines (GPU batches) run at a time (0: as memory allows)."""
        self._lib.fgpu_server_set_max_engines(self._h, int(n))

    def slot_reuse(self, share=-1.0):
        """Sets the share of an engine's models that must have finished before
        its running models move into a new engine with waiting requests (0:
        never; < 0: unchanged); returns the number of such moves so far."""
        n = ctypes.c_longlong(0)
        self._lib.fgpu_server_slot_reuse(self._h, float(share), ctypes.byref(n))
        return n.value

    def status(self):
        s = np.zeros(4, dtype=np.int64)
        self._lib.fgpu_server_status(self._h, _ptr(s, ctypes.c_longlong))
        return {"requests": int(s[0]), "pending": int(s[1]), "live_batches": int(s[2]), "bytes": int(s[3])}

    def request(self, rid):
        st = ctypes.c_int()
        t = np.zeros(3)
        it, steps = ctypes.c_longlong(), ctypes.c_longlong()
        self._lib.fgpu_server_request(self._h, rid, ctypes.byref(st), _ptr(t, ctypes.c_double), ctypes.byref(it),
                                      ctypes.byref(steps))
        return {"state": st.value, "arrival": t[0], "admitted": t[1], "finished": t[2], "iterations": it.value,
                "steps": steps.value}

    def result(self, rid):
        m = self._models[rid]
        ur = np.zeros(12 * m.ntri)
        if self._lib.fgpu_server_result(self._h, rid, _ptr(ur, ctypes.c_double)) != 0:
            raise FedemException("result: " + self._lib.fgpu_last_error().decode())
        return ur.reshape((-1, 4, 3)).transpose(0, 2, 1)
