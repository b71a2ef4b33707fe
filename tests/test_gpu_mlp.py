"""The closure network's tensor-core kernels (bl_mlp.cu) against the CPU
reference (oracle/mlp.py): forward values and loss gradients agree with the
reference that rounds the same operands to BF16 (to FP32 summation order),
and with the unrounded FP64 network within BF16 accuracy; training lowers
the loss of a learnable target."""
import ctypes as ct

import numpy as np
import pytest

from oracle import mlp

pytestmark = pytest.mark.gpu


def _lib():
    from bookleaf_f90_gb300 import _lib
    return _lib.load()


def _fp(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Net:
    def __init__(self, params):
        self.L = _lib()
        self.m = ct.c_void_p()
        p = _fp(params)
        assert self.L.bl_mlp_create(ct.byref(self.m), p.ctypes.data_as(ct.c_void_p)) == 0

    def predict(self, x):
        x = _fp(x)
        y = np.zeros((len(x), mlp.NO), np.float32)
        assert self.L.bl_mlp_predict(self.m, x.ctypes.data_as(ct.c_void_p), len(x),
                                     y.ctypes.data_as(ct.c_void_p)) == 0
        return y

    def gradient(self, x, t):
        x, t = _fp(x), _fp(t)
        g = np.zeros(mlp.NPARAM, np.float32)
        loss = ct.c_float(0)
        assert self.L.bl_mlp_gradient(self.m, x.ctypes.data_as(ct.c_void_p),
                                      t.ctypes.data_as(ct.c_void_p), len(x),
                                      g.ctypes.data_as(ct.c_void_p), ct.byref(loss)) == 0
        return loss.value, g

    def params(self):
        p = np.zeros(mlp.NPARAM, np.float32)
        assert self.L.bl_mlp_params(self.m, p.ctypes.data_as(ct.c_void_p)) == 0
        return p

    def close(self):
        self.L.bl_mlp_destroy(self.m)


def _data(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(0, 1, (n, mlp.NI)), rng.normal(0, 1, (n, mlp.NO))


def test_forward_matches_reference():
    p = mlp.init_params(seed=2)
    x, _ = _data(1000, 5)            # 1000 = 15 blocks of 64 + a part-filled one
    net = Net(p)
    y = net.predict(x)
    ref, _ = mlp.forward(p, _fp(x), bf=True)
    ref64, _ = mlp.forward(p, x)
    scale = np.max(np.abs(ref64))
    assert np.max(np.abs(y - ref)) <= 2e-3 * scale
    assert np.max(np.abs(y - ref64)) <= 3e-2 * scale
    net.close()


def test_gradient_matches_reference():
    p = mlp.init_params(seed=4)
    x, t = _data(777, 6)
    net = Net(p)
    loss, g = net.gradient(x, t)
    lref, gref = mlp.gradient(p, _fp(x), _fp(t), bf=True)
    l64, g64 = mlp.gradient(p, x, t)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    assert np.linalg.norm(g - gref) <= 1e-3 * np.linalg.norm(gref)
    assert np.linalg.norm(g - g64) <= 3e-2 * np.linalg.norm(g64)
    # layer by layer, so that an indexing slip in one block cannot hide
    k = 0
    for name, shape in mlp.SHAPES:
        n = int(np.prod(shape))
        a, b = g[k:k + n], gref[k:k + n]
        assert np.linalg.norm(a - b) <= 2e-3 * np.linalg.norm(b) + 1e-9, name
        k += n
    net.close()


def test_training_learns_a_teacher_network():
    teacher = mlp.init_params(seed=11)
    x, _ = _data(8192, 12)
    t, _ = mlp.forward(teacher, x)
    net = Net(mlp.init_params(seed=13))
    l0, _ = net.gradient(x, t)
    losses = np.zeros(40, np.float32)
    xf, tf = _fp(x), _fp(t)
    assert net.L.bl_mlp_train(net.m, xf.ctypes.data_as(ct.c_void_p), tf.ctypes.data_as(ct.c_void_p),
                              len(x), 40, 512, ct.c_float(3e-3), 7,
                              losses.ctypes.data_as(ct.c_void_p)) == 0
    l1, _ = net.gradient(x, t)
    assert l1 < 0.05 * l0, (l0, l1, losses[:5], losses[-5:])
    assert losses[-1] < losses[0]
    net.close()
