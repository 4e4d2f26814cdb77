"""ctypes wrapper of oracle/cpu_ref.cpp (TEST INFRASTRUCTURE: the large-N oracle
and the timed CPU baseline; see that file's header)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_ref.cpp")
LIB = os.path.join(HERE, "_build", "libcpuref.so")
_lib = None

KIND = {"matern12": 1, "matern32": 2, "matern52": 3, "matern72": 4}
LIK = {"gaussian": 1, "logit": 2, "probit": 3, "poisson": 4, "hetero_exp": 5, "hetero_softplus": 6}


def build():
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) > os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        d, i32, i64 = ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int64
        ip = ctypes.POINTER(ctypes.c_int)
        lib.cpuref_step.argtypes = [i64, i32, i32, ip, d, d, i32, ctypes.c_double, i32, i32, ctypes.c_double,
                                    d, d, d, d, d, d, d, d, d, i32, d]
        lib.cpuref_step.restype = ctypes.c_int
        lib.cpuref_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class CpuRefModel:
    """Float64 sequential Markov VI GP (one series) with the same state layout as
    the CUDA library: components = [(kind, variance, lengthscale)], combine 0 =
    Sum, 1 = Independent."""

    def __init__(self, components, combine, lik, x, y, lik_variance=1.0, num_cub=20, threads=0):
        self.lib = load()
        ind = np.argsort(np.asarray(x, dtype=np.float64), kind="stable")
        x = np.asarray(x, dtype=np.float64)[ind]
        self.y = np.ascontiguousarray(np.asarray(y, dtype=np.float64)[ind])
        self.dt = np.ascontiguousarray(np.concatenate([[0.0], np.diff(x)]))
        self.N = x.shape[0]
        self.nc = len(components)
        self.kind = (ctypes.c_int * self.nc)(*[KIND[c[0]] for c in components])
        self.var = np.array([c[1] for c in components], dtype=np.float64)
        self.ell = np.array([c[2] for c in components], dtype=np.float64)
        self.combine = combine
        self.P = self.nc if combine else 1
        P, N = self.P, self.N
        self.lik, self.lik_variance, self.num_cub = LIK[lik], lik_variance, num_cub
        self.threads = threads
        self.nat1 = np.zeros([N, P])
        self.nat2 = np.tile(1e-2 * np.eye(P), [N, 1, 1])
        self.pm = np.zeros([N, P])
        self.pv = np.tile(np.eye(P), [N, 1, 1])
        self.grad = np.zeros([N, P])
        self.hess = np.zeros([N, P, P])
        self.lin = np.zeros([N, P])
        self.result = np.zeros(4)
        self.step(newton=False)

    def step(self, newton=True, lr=1.0):
        rc = self.lib.cpuref_step(self.N, self.nc, self.combine, self.kind, _p(self.var), _p(self.ell), self.lik,
                                  self.lik_variance, self.num_cub, 1 if newton else 0, lr, _p(self.dt), _p(self.y),
                                  _p(self.nat1), _p(self.nat2), _p(self.pm), _p(self.pv), _p(self.grad),
                                  _p(self.hess), _p(self.lin), int(self.threads), _p(self.result))
        if rc != 0:
            raise ValueError("cpuref_step rejected its arguments")
        return self.result[0]

    @property
    def energy(self):
        return self.result[0]
