"""Learned start vectors: the sed_mlp_* entry points of libsed.

The reference starts PRIMME from its own random vector (src/SpinED.hs:385-394).
Here a ground state computed at a neighbouring coupling (or several) is
sampled into training data, a small BF16 MLP is trained on the GPU by the
library's own forward and backward kernels, and the network's amplitudes over
the new basis become the Krylov start vector (``sed_eigh`` with
``SED_START_GIVEN``). Random start and warm start stay available beside it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .internal import SpinBasis as Basis, _Handle, _mk, check_status, get_number_states


def _ptr(a) -> C.c_void_p:
    """Pointer of a numpy array or a CUDA tensor (anything with data_ptr())."""
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data)
    return C.c_void_p(a.data_ptr())


@dataclass
class Samples:
    states: np.ndarray  # uint64 representatives
    t_abs: np.ndarray   # float32 log|psi(configuration)|
    t_sign: np.ndarray  # float32 1 if psi_r > 0 else 0

    def __len__(self) -> int:
        return len(self.states)

    @staticmethod
    def concat(parts: "list[Samples]") -> "Samples":
        return Samples(np.concatenate([p.states for p in parts]), np.concatenate([p.t_abs for p in parts]),
                       np.concatenate([p.t_sign for p in parts]))


def sample(basis: Basis, psi, n: int, seed: int = 0, sign_mask: int = 0) -> Samples:
    """n representatives drawn with probability psi_r^2 (psi real, host or
    device); psi's global sign is fixed against the sign prior of sign_mask."""
    if isinstance(psi, np.ndarray):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
    out = Samples(np.zeros(n, np.uint64), np.zeros(n, np.float32), np.zeros(n, np.float32))
    check_status(L.load().sed_mlp_sample(basis.ptr, _ptr(psi), n, seed, sign_mask, _ptr(out.states), _ptr(out.t_abs),
                                         _ptr(out.t_sign)))
    return out


class Mlp(_Handle):
    """n_inputs -> hidden -> hidden -> 2 network (see sed_mlp_create)."""
    _destroy = "sed_mlp_destroy"

    def __init__(self, n_inputs: int, hidden: int = 512, sign_mask: int = 0, seed: int = 0):
        super().__init__(_mk(L.load().sed_mlp_create, n_inputs, hidden, sign_mask, seed))
        self.n_inputs, self.hidden, self.sign_mask = n_inputs, hidden, sign_mask

    @property
    def num_params(self) -> int:
        return L.load().sed_mlp_num_params(self.ptr)

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check_status(L.load().sed_mlp_get_params(self.ptr, _ptr(out)))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (self.num_params,)
        check_status(L.load().sed_mlp_set_params(self.ptr, _ptr(p)))

    def unpack(self, p: np.ndarray) -> dict:
        """Split a parameter blob into W1, b1, W2, b2, W3, b3."""
        n, h = self.n_inputs, self.hidden
        sizes = [("W1", (h, n)), ("b1", (h,)), ("W2", (h, h)), ("b2", (h,)), ("W3", (2, h)), ("b3", (2,))]
        out, o = {}, 0
        for name, shp in sizes:
            k = int(np.prod(shp))
            out[name] = p[o:o + k].reshape(shp)
            o += k
        return out

    def set_path(self, path: int) -> None:
        """L.SED_MLP_PATH_AUTO (tensor cores where the shape allows) or
        L.SED_MLP_PATH_SIMT (CUDA cores, FP32 activations)."""
        check_status(L.load().sed_mlp_set_path(self.ptr, path))

    @property
    def uses_tensor_cores(self) -> bool:
        return bool(L.load().sed_mlp_uses_tensor_cores(self.ptr))

    def forward(self, states: np.ndarray) -> np.ndarray:
        states = np.ascontiguousarray(states, dtype=np.uint64)
        out = np.zeros((len(states), 2), np.float32)
        check_status(L.load().sed_mlp_forward(self.ptr, _ptr(states), len(states), _ptr(out)))
        return out

    def loss_grad(self, s: Samples) -> tuple[float, np.ndarray]:
        loss = C.c_double()
        g = np.zeros(self.num_params, np.float32)
        check_status(L.load().sed_mlp_loss_grad(self.ptr, _ptr(s.states), _ptr(s.t_abs), _ptr(s.t_sign), len(s),
                                                C.byref(loss), _ptr(g)))
        return loss.value, g

    def train(self, s: Samples, epochs: int = 4, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_double()
        check_status(L.load().sed_mlp_train(self.ptr, _ptr(s.states), _ptr(s.t_abs), _ptr(s.t_sign), len(s),
                                            epochs, batch, lr, seed, C.byref(loss)))
        return loss.value

    def train_decayed(self, s: Samples, epochs: int, batch: int = 4096, lr: float = 3e-3, seed: int = 0) -> float:
        """Three phases of Adam with a falling learning rate: epochs/2 at lr,
        epochs/4 at lr/3 and the rest at lr/15 (each phase reshuffles from
        its own seed); returns the loss of the last batch."""
        e1 = max(1, epochs // 2)
        e2 = max(0, epochs // 4)
        e3 = max(0, epochs - e1 - e2)
        loss = self.train(s, epochs=e1, batch=batch, lr=lr, seed=seed)
        for k, (e, f) in enumerate(((e2, 1 / 3), (e3, 1 / 15))):
            if e:
                loss = self.train(s, epochs=e, batch=batch, lr=lr * f, seed=seed + 1 + k)
        return loss

    def start_vector(self, basis: Basis, out=None):
        """Start vector over the basis (numpy array, or fills a CUDA tensor)."""
        if out is None:
            out = np.zeros(get_number_states(basis), np.float64)
        check_status(L.load().sed_mlp_start_vector(self.ptr, basis.ptr, _ptr(out)))
        return out


class PatchMlp(Mlp):
    """Size-independent network (sed_mlp_create_patch): the MLP applied to
    every site's patch of spins and summed over the sites. `patches` is an
    (n_sites, P) integer array of site indices; `rebind` moves the trained
    network to another lattice with the same patch shape."""

    def __init__(self, patches, hidden: int = 128, sign_mask: int = 0, seed: int = 0):
        t = np.ascontiguousarray(patches, dtype=np.uint16)
        n, P = t.shape
        _Handle.__init__(self, _mk(L.load().sed_mlp_create_patch, n, P, C.c_void_p(t.ctypes.data), hidden,
                                   sign_mask, seed))
        self.n_inputs, self.hidden, self.sign_mask, self.n_sites = P, hidden, sign_mask, n

    def rebind(self, patches, sign_mask: int = 0) -> None:
        t = np.ascontiguousarray(patches, dtype=np.uint16)
        assert t.shape[1] == self.n_inputs, "the patch shape must stay the same"
        check_status(L.load().sed_mlp_set_patch_sites(self.ptr, t.shape[0], C.c_void_p(t.ctypes.data), sign_mask))
        self.n_sites, self.sign_mask = t.shape[0], sign_mask

