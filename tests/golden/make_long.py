"""Generate the long-run golden digests in this folder from the reference itself.

Runs the reference's own serial FP64 step (oracle/_ref/ref_harness, built from
the reference sources by oracle/build_ref.sh) for each benchmark
configuration's whole step count, and stores a digest of the end state
(model_gb300/digest.py: random projections, level norms and a point sample of
u, v, w, theta, (qv, qc, qr,) pi) with the generator that rebuilds the initial
state:

  long_thunderstorm.npz      128x128x48 Kessler thunderstorm, 600 steps
  long_monsoon_vortex.npz    192x128x32 ITCZ-shear monsoon vortex, 500 steps
  long_member_small.npz      ensemble member 0 (96x96x40), 300 steps
  long_member_large.npz      ensemble member 64 (160x160x48), 300 steps
  long_squall_line.npz       512x512x64 squall line, 10 of its 400 steps
                             (one host core needs about 40 s per step)

The cases run in parallel, one process each.  Usage (where the reference
sources exist):  python tests/golden/make_long.py [case ...]
"""
from __future__ import annotations

import json
import os
import sys
import time
from concurrent.futures import ProcessPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from model_gb300 import abi, configs, digest  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

# name -> (generator, kwargs, steps)
CASES = {
    "thunderstorm": ("thunderstorm", {}, 600),
    "monsoon_vortex": ("monsoon_vortex", {}, 500),
    "member_small": ("ensemble_member", {"m": 0, "nx": 96, "ny": 96, "nz": 40}, 300),
    "member_large": ("ensemble_member", {"m": 64, "nx": 160, "ny": 160, "nz": 48}, 300),
    "squall_line": ("squall_line", {}, 10),
}


def make_workload(gen: str, kw: dict):
    return getattr(configs, gen)(**kw)


def end_state_fields(wl, dump: dict) -> dict:
    names = ["u", "v", "w", "th"] + (["qv", "qc", "qr"] if wl.microphysics_option else [])
    out = {k: dump[k] for k in names}
    out["pi"] = dump["pi"]
    return out


def run_case(name: str) -> str:
    from oracle import oracle as O
    gen, kw, steps = CASES[name]
    wl = make_workload(gen, kw)
    t0 = time.time()
    dump = O.run_reference(wl, "run", steps)
    el = time.time() - t0
    shape = (wl.nx, wl.ny, wl.nz)
    d = digest.digest(end_state_fields(wl, dump), shape, m=64 if wl.points < 4_000_000 else 32)
    d["generator"] = np.array(gen)
    d["kwargs"] = np.array(json.dumps(kw))
    d["steps"] = np.int64(steps)
    d["grid"] = np.array(shape, dtype=np.int64)
    d["input_norms"] = np.array([np.linalg.norm(np.asarray(wl.fields[k], dtype=np.float64))
                                 for k in sorted(wl.fields)])
    d["input_names"] = np.array(json.dumps(sorted(wl.fields)))
    d["reference_seconds"] = np.float64(el)
    path = os.path.join(HERE, f"long_{name}.npz")
    np.savez_compressed(path, **d)
    return f"wrote {path} ({os.path.getsize(path)} bytes, reference {el:.0f} s for {steps} steps)"


def main():
    names = sys.argv[1:] or list(CASES)
    with ProcessPoolExecutor(max_workers=len(names)) as ex:
        for msg in ex.map(run_case, names):
            print(msg, flush=True)


if __name__ == "__main__":
    main()
