"""Trains the learned coarse space of the FGMRES preconditioner and writes
its parameters (``python -m mbem_gb300.la.train_learned [out.npy]``).

Training set: six cubes (12 or 16 squares per face) with a FAULT_TRACTION
fault of 8 to 16 squares per side, each at a dip drawn uniformly in
[30, 90] degrees (seeded), 3400 block-Jacobi errors per mesh from direct
dense solves (about 20,000 pairs); 3000 Adam steps of 64 errors. The
parameters shipped in ``mbem_gb300/data/learned_coarse.npy`` come from this
script on one GB300.
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

TRAINING_MESHES = [(12, 8), (16, 12), (12, 10), (16, 8), (16, 16), (12, 12)]
SAMPLES_PER_MESH = 3400
STEPS = 3000
BATCH = 64
LR = 2e-3

DEFAULT_PARAMS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data",
                              "learned_coarse.npy")


def load_default() -> np.ndarray:
    """The shipped trained parameters (FP32, MBEM_NN_PARAMS)."""
    return np.load(DEFAULT_PARAMS).astype(np.float32)


def main(out: str = DEFAULT_PARAMS, verbose: bool = True) -> np.ndarray:
    import torch

    from ..backends.dense import DenseBackend
    from ..cases import fault_traction_model
    from ..model import generate_system
    from .learned import TrainingMesh, train

    backend = DenseBackend(jump="calibrated", deflate=True)
    rng = np.random.default_rng(0)
    meshes = []
    t0 = time.time()
    for n_face, n_fault in TRAINING_MESHES:
        dip = float(rng.uniform(30, 90))
        model, eps = fault_traction_model(n_face, n_fault, dip)
        asm = backend.assemble(generate_system(model), eps)
        meshes.append(TrainingMesh(asm, SAMPLES_PER_MESH, seed=n_face * 100 + n_fault))
        if verbose:
            print(f"training mesh n={n_face} fault={n_fault} dip={dip:.1f} N={asm.b.shape[0]} "
                  f"({time.time() - t0:.1f} s)", flush=True)
        del asm
    params, tr = train(meshes, steps=STEPS, batch=BATCH, lr=LR, log_every=500)
    torch.cuda.synchronize()
    if verbose:
        print("loss history", [(i, round(v, 4)) for i, v in tr.history], flush=True)
    np.save(out, params)
    return params


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_PARAMS)
