"""Pin the beta-plane configuration at its stated length by running the reference core itself: 1024 x 512 cells of
5 km, f0 = 1e-4, beta = 1.6e-11, g = 9.81, H = 100 m, the zonal jet u = 20 sech^2(y / 100 km) in geostrophic balance
plus seeded white-noise height of 0.1 m rms (the project's generator), RK4 with dt = 60 s for 5000 steps
(cpp/plane.cpp:143-189). The reference's cpp/plane.cpp, built by oracle/Makefile without FMA contraction
(oracle/_ref/libref.so), runs Plane::run and the fixture keeps SHA-256 digests of the little-endian FP64 bytes of
h, u and v after 1000 and 5000 steps, the invariants, and a few field values. It runs where the reference checkout
exists (about 15 minutes on one core); the fixture it writes is committed so the tests need no reference.

    python tests/golden/make_plane_config1.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from oracle_lib import OraclePlane, RefPlane, build_oracle, ref_available  # noqa: E402

NX, NY, DX = 1024, 512, 5000.0
PARAMS = dict(f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
JET = (20.0, 1.0e5, 0.1, 1)  # u0, width, noise rms, seed
DT, CHECKPOINTS = 60.0, (1000, 5000)
OUT = os.path.join(HERE, "plane_config1_5000.json")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def initial_state():
    gen = OraclePlane(NX, NY, NX * DX, NY * DX, **PARAMS)
    h, u = gen.jet_grids(*JET)
    return h, u, np.zeros((NY + 1, NX))


def main() -> None:
    build_oracle(with_ref=True)
    if not ref_available():
        sys.exit("the reference checkout is absent: the committed fixture stands")
    h, u, v = initial_state()
    r = RefPlane(NX, NY, NX * DX, NY * DX, **PARAMS)
    r.set(h, u, v)
    out = {"nx": NX, "ny": NY, "dx": DX, "params": PARAMS, "jet": list(JET), "dt": DT,
           "initial": {"h": digest(h), "u": digest(u), "v": digest(v)}, "checkpoints": []}
    done, t0 = 0, time.time()
    for n in CHECKPOINTS:
        r.run((n - done) * DT, DT)
        done = n
        hh, uu, vv = r.get()
        out["checkpoints"].append({"steps": n, "h": digest(hh), "u": digest(uu), "v": digest(vv), "diagnostics": r.diagnostics(),
                                   "samples": {"h[256,512]": hh[256, 512], "u[128,100]": uu[128, 100], "v[300,700]": vv[300, 700]}})
        print(f"{n} steps ({time.time() - t0:.0f} s)", flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
