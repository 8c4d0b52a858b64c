"""Float64 oracle states at the workloads' full sizes, stored on a sub-lattice.

    python tests/golden/make_large_parity.py [tgv128|tgv256|khi|khi4k] ...

Runs the oracle (``oracle/spectral.py``, the NumPy float64 restatement of the
reference pinned to the reference's own outputs by tests/test_oracle_golden.py)
with ``fused=True``: one spectral sum per stage, the same operator as the
reference's per-derivative full transforms up to rounding.  The initial
states are rounded to float32 first, as the float32 engine receives them.

Writes tests/golden/tgv3d_{128,256}_200.npz, tests/golden/khi_c4_t1.npz and
tests/golden/khi2d_4k_steps.npz (the reference's khi2d problem on its shipped
3840 x 2160 grid, a few CFL steps).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))

from oracle import spectral as O  # noqa: E402
from phrike_gb300 import problems  # noqa: E402
import parity_cases as PC  # noqa: E402


def tgv(n: int) -> None:
    U = problems.taylor_green_3d(n).astype(np.float32).astype(np.float64)
    s = O.EulerSolver(O.FourierBox((n, n, n), (2 * np.pi,) * 3, dealias=True), cfl=0.25, fused=True)
    t0 = time.time()
    for i in range(PC.TGV_STEPS):
        U = s.step(U, PC.TGV_DT)
        if i % 20 == 0:
            print(f"tgv{n} step {i} {time.time() - t0:.0f}s", flush=True)
    st = PC.TGV_STRIDE[n]
    np.savez_compressed(os.path.join(HERE, f"tgv3d_{n}_200.npz"), U=PC.sub(U, st), stride=st,
                        steps=PC.TGV_STEPS, dt=PC.TGV_DT, cons=np.array(list(O.conserved_sums(U, 1.4).values())))


def khi() -> None:
    out = {}
    for n, (idx, u0, amp) in PC.khi_samples().items():
        U0 = problems.kelvin_helmholtz_2d(n, n, U0=u0, A=amp).astype(np.float32).astype(np.float64)
        s = O.EulerSolver(O.FourierBox((n, n), (1.0, 1.0), dealias=True), cfl=PC.KHI_CFL, fused=True)
        t0 = time.time()
        U, t, dts = s.run(U0, 0.0, PC.KHI_T_END)
        print(f"khi{n}: {len(dts)} steps, t={t}, {time.time() - t0:.0f}s", flush=True)
        st = PC.KHI_STRIDE[n]
        out[f"n{n}_U"] = PC.sub(U, st)
        out[f"n{n}_stride"] = st
        out[f"n{n}_steps"] = len(dts)
        out[f"n{n}_index"] = idx
        out[f"n{n}_u0"] = u0
        out[f"n{n}_amp"] = amp
    np.savez_compressed(os.path.join(HERE, "khi_c4_t1.npz"), **out)


def khi4k() -> None:
    cfg = PC.khi4k_config()
    U = PC.khi4k_initial_state(cfg).astype(np.float32).astype(np.float64)
    g = cfg["grid"]
    sf = cfg["integration"]["spectral_filter"]
    box = O.FourierBox((int(g["Ny"]), int(g["Nx"])), (float(g["Ly"]), float(g["Lx"])), dealias=True,
                       filter_enabled=True, filter_p=int(sf["p"]), filter_alpha=float(sf["alpha"]))
    s = O.EulerSolver(box, gamma=float(cfg["physics"]["gamma"]), cfl=float(cfg["integration"]["cfl"]), fused=True)
    dts = []
    t0 = time.time()
    for i in range(PC.KHI4K_STEPS):
        dt = s.compute_dt(U)
        U = s.step(U, dt)
        dts.append(dt)
        print(f"khi4k step {i} dt={dt:.3e} {time.time() - t0:.0f}s", flush=True)
    st = PC.KHI4K_STRIDE
    np.savez_compressed(os.path.join(HERE, "khi2d_4k_steps.npz"), U=PC.sub(U, st), stride=st, dts=np.array(dts))


if __name__ == "__main__":
    for what in sys.argv[1:] or ["tgv128", "tgv256", "khi", "khi4k"]:
        if what == "khi4k":
            khi4k()
        elif what == "khi":
            khi()
        else:
            tgv(int(what[3:]))
