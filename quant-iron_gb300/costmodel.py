"""The learned fusion cost model (C ABI qi_costmodel_*; kernels in csrc/qi_mlp.cu).

collect(n, count, seed)        engine-measured timings of random device ops -> (X, y)
train(X, y, epochs, lr, seed)  full-batch Adam on the GPU; becomes the process-wide model
predict(X)                     y = log(ms per 2^28 amplitudes)
loss_and_gradient(X, y)        MSE and its gradient (flat parameter vector)
params() / set_params(p)       save / restore the model
"""
import ctypes

import numpy as np

from ._abi import COSTMODEL_FEATURES, check, lib

_pf = ctypes.POINTER(ctypes.c_float)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def num_params():
    n = ctypes.c_int64()
    check(lib.qi_costmodel_num_params(ctypes.byref(n)))
    return n.value


def collect(num_qubits, count, seed=0):
    X = np.zeros((count, COSTMODEL_FEATURES), dtype=np.float32)
    y = np.zeros(count, dtype=np.float32)
    check(lib.qi_costmodel_collect(int(num_qubits), int(count), int(seed), X.ctypes.data_as(_pf), y.ctypes.data_as(_pf)))
    return X, y


def train(X, y, epochs=2000, lr=3e-3, seed=0):
    X, y = _f32(X), _f32(y)
    hist = np.zeros(epochs, dtype=np.float32)
    check(lib.qi_costmodel_train(X.ctypes.data_as(_pf), y.ctypes.data_as(_pf), y.size, int(epochs), float(lr),
                                 int(seed), hist.ctypes.data_as(_pf)))
    return hist


def predict(X):
    X = _f32(X)
    out = np.zeros(X.shape[0], dtype=np.float32)
    check(lib.qi_costmodel_predict(X.ctypes.data_as(_pf), X.shape[0], out.ctypes.data_as(_pf)))
    return out


def loss_and_gradient(X, y):
    X, y = _f32(X), _f32(y)
    loss = ctypes.c_float()
    g = np.zeros(num_params(), dtype=np.float32)
    check(lib.qi_costmodel_loss_and_gradient(X.ctypes.data_as(_pf), y.ctypes.data_as(_pf), y.size, ctypes.byref(loss),
                                             g.ctypes.data_as(_pf)))
    return float(loss.value), g


def init(seed=0):
    check(lib.qi_costmodel_init(int(seed)))


def params():
    p = np.zeros(num_params(), dtype=np.float32)
    trained = ctypes.c_int32()
    check(lib.qi_costmodel_get_params(p.ctypes.data_as(_pf), p.size, ctypes.byref(trained)))
    return p, bool(trained.value)


def set_params(p, trained=True):
    p = _f32(p)
    check(lib.qi_costmodel_set_params(p.ctypes.data_as(_pf), p.size, 1 if trained else 0))
