"""ctypes view of the learned pair-energy surrogate (include/cgppd_surrogate.h).

Thin: argument marshalling only; training, inference and screening run in the native
library on the GPU.
"""
import ctypes

import numpy as np

from . import CgppdError, check, lib

c_int, c_float, c_double, c_void_p = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p
c_ll, c_ull = ctypes.c_longlong, ctypes.c_ulonglong
P = ctypes.POINTER

N_IN = 8
HIDDEN = 256

_DECL = {
    "cgppd_surrogate_create": (c_void_p, [c_int, c_ull]),
    "cgppd_surrogate_destroy": (None, [c_void_p]),
    "cgppd_surrogate_num_params": (c_int, []),
    "cgppd_surrogate_get_params": (c_int, [c_void_p, P(c_float)]),
    "cgppd_surrogate_set_params": (c_int, [c_void_p, P(c_float)]),
    "cgppd_surrogate_loss_grad": (c_int, [c_void_p, P(c_float), P(c_float), c_int, P(c_float), P(c_float)]),
    "cgppd_surrogate_predict": (c_int, [c_void_p, c_void_p, c_int, P(c_float)]),
    "cgppd_surrogate_add_samples": (c_int, [c_void_p, P(c_float), P(c_float), c_int]),
    "cgppd_surrogate_clear_samples": (c_int, [c_void_p]),
    "cgppd_surrogate_num_samples": (c_ll, [c_void_p]),
    "cgppd_surrogate_get_samples": (c_int, [c_void_p, P(c_float), P(c_float), c_ll]),
    "cgppd_surrogate_collect": (c_int, [c_void_p, c_void_p, c_int, c_int, c_double, c_ull]),
    "cgppd_surrogate_train": (c_int, [c_void_p, c_int, c_float, c_float, c_float, P(c_float)]),
    "cgppd_engine_surrogate_compatible": (c_int, [c_void_p, c_int]),
    "cgppd_engine_set_surrogate": (c_int, [c_void_p, c_void_p, c_float, c_float, c_int]),
    "cgppd_engine_surrogate_stats": (c_int, [c_void_p, c_int, P(c_double)]),
}


def _L():
    L = lib()
    if not getattr(L, "_surrogate_declared", False):
        for name, (res, args) in _DECL.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L._surrogate_declared = True
    return L


def _ok(rc, where):
    if rc < 0:
        check(where)
        raise CgppdError(where + " failed")
    return rc


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _pf(a):
    return a.ctypes.data_as(P(c_float))


# offsets of the FP32 master parameters
OFF = {}
_o = 0
for _name, _size in (("W1", HIDDEN * N_IN), ("b1", HIDDEN), ("W2", HIDDEN * HIDDEN), ("b2", HIDDEN),
                     ("W3", HIDDEN * HIDDEN), ("b3", HIDDEN), ("W4", HIDDEN * HIDDEN), ("b4", HIDDEN),
                     ("w5", HIDDEN), ("b5", 1)):
    OFF[_name] = (_o, _size)
    _o += _size
N_PARAMS = _o


def unpack(flat):
    """Parameter vector -> dict of arrays (W as [out][in])."""
    out = {}
    for k, (o, n) in OFF.items():
        v = np.asarray(flat[o:o + n])
        if k == "W1":
            v = v.reshape(HIDDEN, N_IN)
        elif k in ("W2", "W3", "W4"):
            v = v.reshape(HIDDEN, HIDDEN)
        out[k] = v
    return out


class Surrogate:
    """MLP 8 -> 256 x 4 (SiLU) -> 1 predicting a rigid pair's inter-molecule energy."""

    def __init__(self, batch=8192, seed=20261203):
        L = _L()
        assert L.cgppd_surrogate_num_params() == N_PARAMS
        h = L.cgppd_surrogate_create(int(batch), c_ull(seed))
        if not h:
            check("cgppd_surrogate_create")
            raise CgppdError("cgppd_surrogate_create failed")
        self.h = h
        self.batch = batch

    def close(self):
        if getattr(self, "h", None):
            _L().cgppd_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        p = np.zeros(N_PARAMS, np.float32)
        _ok(_L().cgppd_surrogate_get_params(self.h, _pf(p)), "get_params")
        return p

    @params.setter
    def params(self, p):
        p = _f32(p)
        assert p.size == N_PARAMS
        _ok(_L().cgppd_surrogate_set_params(self.h, _pf(p)), "set_params")

    def loss_grad(self, X, y, grad=True):
        X, y = _f32(X), _f32(y)
        loss = c_float(0)
        g = np.zeros(N_PARAMS, np.float32) if grad else None
        _ok(_L().cgppd_surrogate_loss_grad(self.h, _pf(X), _pf(y), len(y), ctypes.byref(loss),
                                           _pf(g) if grad else None), "loss_grad")
        return float(loss.value), g

    def predict(self, X):
        X = _f32(X)
        out = np.zeros(len(X), np.float32)
        _ok(_L().cgppd_surrogate_predict(self.h, X.ctypes.data, len(X), _pf(out)), "predict")
        return out

    def add_samples(self, X, y):
        X, y = _f32(X), _f32(y)
        _ok(_L().cgppd_surrogate_add_samples(self.h, _pf(X), _pf(y), len(y)), "add_samples")

    def clear_samples(self):
        _ok(_L().cgppd_surrogate_clear_samples(self.h), "clear_samples")

    @property
    def n_samples(self):
        return int(_L().cgppd_surrogate_num_samples(self.h))

    def samples(self):
        n = self.n_samples
        X = np.zeros((n, N_IN), np.float32)
        y = np.zeros(n, np.float32)
        _ok(_L().cgppd_surrogate_get_samples(self.h, _pf(X), _pf(y), n), "get_samples")
        return X, y

    def collect(self, engine, sim, n, proposal_fraction=0.5, seed=1):
        _ok(_L().cgppd_surrogate_collect(self.h, engine.h, int(sim), int(n), float(proposal_fraction), c_ull(seed)),
            "collect")

    def train(self, epochs, lr=1e-3, clip=25.0, val_fraction=0.05):
        hist = np.zeros(2 * max(epochs, 1), np.float32)
        _ok(_L().cgppd_surrogate_train(self.h, int(epochs), float(lr), float(clip), float(val_fraction), _pf(hist)),
            "train")
        return hist[:2 * epochs].reshape(epochs, 2)


def compatible(engine, sim):
    return _ok(_L().cgppd_engine_surrogate_compatible(engine.h, int(sim)), "surrogate_compatible") == 1


def attach(engine, surrogate, rmse_threshold=0.5, error_window=25.0, min_evals=100):
    """Screen `engine`'s compatible simulations with `surrogate` (None detaches);
    returns how many simulations screen."""
    return _ok(_L().cgppd_engine_set_surrogate(engine.h, surrogate.h if surrogate is not None else None,
                                               float(rmse_threshold), float(error_window), int(min_evals)),
               "set_surrogate")


def stats(engine, sim):
    out = np.zeros(7, np.float64)
    _ok(_L().cgppd_engine_surrogate_stats(engine.h, int(sim), out.ctypes.data_as(P(c_double))), "surrogate_stats")
    keys = ("proposals", "stage1_reject", "stage2_eval", "stage2_accept", "sum_e2", "n_e2", "screening")
    d = dict(zip(keys, out.tolist()))
    d["rmse"] = (d["sum_e2"] / d["n_e2"]) ** 0.5 if d["n_e2"] else float("nan")
    return d


def train_on_engine(engine, sim, n_samples, blocks, steps_per_block, epochs, batch=8192, lr=1e-3, clip=25.0,
                    proposal_fraction=0.5, seed=20261203, surrogate=None):
    """The training recipe: run the exact engine for `blocks` blocks, collecting an equal
    share of (pose, exact energy) samples from its replicas after each block, then train.
    Returns (surrogate, history)."""
    s = surrogate or Surrogate(batch=batch, seed=seed)
    per = max(1, n_samples // max(blocks, 1))
    for b in range(blocks):
        engine.run(1, steps_per_block, exchange_after_last=True)
        engine.synchronize()
        s.collect(engine, sim, per, proposal_fraction, seed=seed + 7919 * (b + 1))
    hist = s.train(epochs, lr=lr, clip=clip)
    return s, hist
