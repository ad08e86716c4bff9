"""A numpy-backed stand-in for the parts of `jax` the reference imports.

Used only by `make_golden.py` (in the development container, where the
reference sources are present and JAX is not) to execute the reference's own
modules and record their outputs as fixtures. jax.numpy maps onto numpy,
`jit` is the identity, and `jax.random` draws from numpy generators keyed by
the PRNG key; every draw is appended to `DRAWS` so a fixture can carry the
exact random inputs the reference consumed.
"""
from __future__ import annotations

import hashlib
import sys
import types

import numpy as np

DRAWS: list = []


class JArr(np.ndarray):
    """ndarray with the two jax.Array methods the reference calls."""

    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self


class _At:
    def __init__(self, a):
        self.a = a

    def __getitem__(self, idx):
        return _AtIdx(self.a, idx)


class _AtIdx:
    def __init__(self, a, idx):
        self.a, self.idx = a, idx

    def set(self, v):
        b = np.array(self.a, copy=True)
        b[self.idx] = v
        return b.view(JArr)


def _j(x):
    x = np.asarray(x)
    return x.view(JArr)


def _wrap(fn):
    def f(*a, **k):
        k.pop("precision", None)
        out = fn(*a, **k)
        return _j(out) if isinstance(out, np.ndarray) else out
    return f


def _key_seed(key) -> int:
    h = hashlib.sha256(np.asarray(key, np.uint64).tobytes()).digest()
    return int.from_bytes(h[:8], "little")


def _make_random():
    r = types.ModuleType("jax.random")

    def PRNGKey(seed):
        return np.asarray([0, int(seed) & 0xFFFFFFFF], np.uint64)

    def split(key, num=2):
        s = _key_seed(key)
        return [np.asarray([s & 0xFFFFFFFF, (s >> 32) + i + 1], np.uint64) for i in range(num)]

    def fold_in(key, data):
        s = _key_seed(np.concatenate([np.asarray(key, np.uint64), [np.uint64(int(data))]]))
        return np.asarray([s & 0xFFFFFFFF, s >> 32], np.uint64)

    def normal(key, shape, dtype=np.float32):
        z = np.random.default_rng(_key_seed(key)).standard_normal(shape).astype(dtype)
        DRAWS.append(("normal", z))
        return _j(z)

    def bernoulli(key, p, shape):
        z = np.random.default_rng(_key_seed(key)).random(shape) < p
        DRAWS.append(("bernoulli", z))
        return _j(z)

    r.PRNGKey, r.split, r.fold_in, r.normal, r.bernoulli = PRNGKey, split, fold_in, normal, bernoulli
    return r


def install() -> None:
    jax = types.ModuleType("jax")
    jnp = types.ModuleType("jax.numpy")
    for name in ("complex64", "complex128", "float32", "float64", "int32", "uint32"):
        setattr(jnp, name, getattr(np, name))
    for name in ("abs", "asarray", "concatenate", "real", "sum", "maximum", "max",
                 "sqrt", "stack", "where", "zeros", "zeros_like", "ones", "ones_like",
                 "matmul", "tensordot", "array", "exp", "cos", "sin", "conj", "eye"):
        setattr(jnp, name, _wrap(getattr(np, name)))
    fft = types.ModuleType("jax.numpy.fft")
    fft.ifftn = _wrap(np.fft.ifftn)
    fft.fftn = _wrap(np.fft.fftn)
    jnp.fft = fft
    linalg = types.ModuleType("jax.numpy.linalg")
    linalg.norm = _wrap(np.linalg.norm)
    linalg.eigh = _wrap(np.linalg.eigh)
    jnp.linalg = linalg
    jax.numpy = jnp
    jax.Array = np.ndarray

    def jit(fn=None, **_kw):
        if fn is None:
            return lambda f: f
        return fn
    jax.jit = jit
    lax = types.ModuleType("jax.lax")

    class Precision:
        HIGHEST = "highest"
        DEFAULT = "default"
    lax.Precision = Precision

    def dynamic_update_slice_in_dim(buf, x, start, axis=0):
        b = np.array(buf, copy=True)
        sl = [slice(None)] * b.ndim
        sl[axis] = slice(int(start), int(start) + x.shape[axis])
        b[tuple(sl)] = x
        return _j(b)
    lax.dynamic_update_slice_in_dim = dynamic_update_slice_in_dim
    jax.lax = lax
    jax.random = _make_random()
    jax.local_devices = lambda: []
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.numpy.fft"] = fft
    sys.modules["jax.numpy.linalg"] = linalg
    sys.modules["jax.lax"] = lax
    sys.modules["jax.random"] = jax.random
