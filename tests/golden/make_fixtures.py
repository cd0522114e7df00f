"""Regenerate the golden fixtures under tests/golden/ from the reference.

Run where the reference source tree is present, naming its root:

    FE_GPU_REFERENCE=<reference tree> python tests/golden/make_fixtures.py

reference_generator_small.npz: output of the reference's own synthetic panel
generator (tools/generate_synthetic_data.py, build_panel) at a small size,
used to check that fe_gpu_gb300.synth.reference_panel restates it exactly.
"""
import argparse
import importlib.util
import json
import os
from pathlib import Path

import numpy as np

if not os.environ.get("FE_GPU_REFERENCE"):
    raise SystemExit("set FE_GPU_REFERENCE to the root of the reference source tree")
REF = Path(os.environ["FE_GPU_REFERENCE"])
OUT = Path(__file__).resolve().parent


def load_generator():
    spec = importlib.util.spec_from_file_location("ref_gen", REF / "tools" / "generate_synthetic_data.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    gen = load_generator()
    meta = dict(workers=60, firms=13, periods=7, extra_vars=3, seed=1234)
    args = argparse.Namespace(workers=meta["workers"], firms=meta["firms"], periods=meta["periods"], intercept=1.0,
                              betas=[0.4, -0.2], extra_vars=meta["extra_vars"], extra_coeffs=None, extra_std=0.3,
                              noise_std=0.5, sick_std=0.5, iv_vars=0, iv_noise_std=0.25, endog_cols=None,
                              seed=meta["seed"])
    wages, W, Z, fe_ids, _, names, _ = gen.build_panel(args)
    np.savez_compressed(OUT / "reference_generator_small.npz", y=wages, W=W, fe_ids=fe_ids,
                        coeffs=args.extra_coeffs_actual, meta=json.dumps(meta))
    print("wrote", OUT / "reference_generator_small.npz", wages.shape, W.shape)


if __name__ == "__main__":
    main()
