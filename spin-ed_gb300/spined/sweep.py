"""J1-J2 sweep on the 6x6 torus with three start vectors per point.

For J2/J1 in 0.00, 0.05, ..., 0.60 (nearest bonds J1 = 1, diagonal
next-nearest bonds J2; sector: Hamming weight 18, translations x C4v x spin
inversion, all characters +1) every point is solved three ways, all to
||H psi - E psi|| <= 1e-8:

  random   the plain method: Philox start vector from seed 1234
  warm     the previous point's ground state
  learned  the start-vector MLP (36 -> 256 -> 256 -> 2), trained on the
           tensor cores on configurations sampled from |psi|^2 of the ground
           states of the two previous points (2^19 per point; the same network
           is fine-tuned point after point, 32 epochs with a falling learning
           rate); its tensor-core inference is timed with the solve

The first point has no earlier ground state, so it has no warm or learned
run. The reference has no counterpart: SpinED starts PRIMME from its own
random vector (src/SpinED.hs:385-394).

    python -m spined.sweep [--precision fp64|mixed] [--epochs 32] [--out sweep.json]
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def run(L: int = 6, j2s=None, precision: str = "mixed", epochs: int = 32, per_point: int = 1 << 19,
        hidden: int = 256, lr: float = 3e-3, log=print) -> list[dict]:
    import torch
    from . import _lib as Lb
    from . import internal as I
    from . import lattices
    from .learned import Mlp, Samples, sample
    from .model import build_model

    j2s = list(np.round(np.arange(0.0, 0.601, 0.05), 2)) if j2s is None else list(j2s)
    prec = Lb.SED_PRECISION_MIXED if precision == "mixed" else Lb.SED_PRECISION_FP64
    b = build_model(lattices.heisenberg_square(L))
    D = I.get_number_states(b.basis)
    mask = lattices.square_sublattice_mask(L)
    net = Mlp(L * L, hidden, sign_mask=mask, seed=5)
    psi = torch.empty(D, dtype=torch.float64, device="cuda")
    start = torch.empty(D, dtype=torch.float64, device="cuda")
    prev = None
    data: Samples | None = None
    window: list = []
    rows = []

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, r

    for k, j2 in enumerate(j2s):
        m = lattices.heisenberg_square(L, j2=float(j2))
        terms = [I.mk_interaction(mat, sites) for mat, sites in m.terms]
        op = I.mk_operator(b.basis, terms)
        op.prepare(Lb.SED_FORM_STREAM)
        row = {"j2": float(j2), "D": D}
        t, r = timed(lambda: I.eigh(op, tol=1e-8, out=psi, seed=1234, precision=prec))
        row["random"] = {"seconds": t, "steps": r.iterations, "E0": float(r.eigenvalues[0]),
                         "residual": float(r.residuals[0])}
        e_ref = float(r.eigenvalues[0])
        if prev is not None:
            start.copy_(prev)
            t, r = timed(lambda: I.eigh(op, tol=1e-8, out=psi, start=start, precision=prec))
            row["warm"] = {"seconds": t, "steps": r.iterations, "E0": float(r.eigenvalues[0]),
                           "residual": float(r.residuals[0])}
        if data is not None:
            def learned():  # the solver normalises the start vector itself
                net.start_vector(b.basis, out=start)
                return I.eigh(op, tol=1e-8, out=psi, start=start, precision=prec)
            t, r = timed(learned)
            row["learned"] = {"seconds": t, "steps": r.iterations, "E0": float(r.eigenvalues[0]),
                              "residual": float(r.residuals[0])}
        for key in ("warm", "learned"):
            if key in row:
                row[key]["eigenvalue_rel_err"] = abs(row[key]["E0"] - e_ref) / abs(e_ref)
        # this point's ground state feeds the next point
        prev = psi.clone()
        if k + 1 < len(j2s):
            t_s, new = timed(lambda: sample(b.basis, prev, per_point, seed=100 + k, sign_mask=mask))
            window = (window + [new])[-2:]
            data = Samples.concat(window)
            t_tr, loss = timed(lambda: net.train_decayed(data, epochs=epochs, batch=4096, lr=lr, seed=100 * k))
            row["training"] = {"samples": len(data), "sample_s": t_s, "train_s": t_tr, "final_loss": loss}
        rows.append(row)
        log(json.dumps(row))
        del op
    return rows


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--epochs", type=int, default=32)
    ap.add_argument("--side", type=int, default=6)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    rows = run(L=a.side, precision=a.precision, epochs=a.epochs, log=lambda s: print(s, flush=True))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rows, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
