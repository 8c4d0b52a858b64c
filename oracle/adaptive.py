"""CPU oracle for adaptive embedded Runge-Kutta time stepping.

TEST INFRASTRUCTURE ONLY.  Restates, in NumPy float64, the reference's
adaptive path (phrike/adaptive.py:22-437) and the solver hooks that drive it:

* the embedded tableaux: Bogacki-Shampine "rk23" (adaptive.py:136-187),
  Dormand-Prince "rk45" (190-238) and the reference's simplified 8-stage
  "rk78" (241-292), kept exactly as the reference defines it;
* the step controller (adaptive.py:23-81): tol = atol + rtol * scale,
  accept when err <= tol, dt_new = dt * clip(safety * (tol/err)^(1/order),
  min_factor, max_factor) with order = the embedded (low) order, and
  dt * max_factor when err == 0;
* the stepper (adaptive.py:341-419): err = max |U_high - U_low|, a
  consecutive-rejection counter, forced acceptance after max_rejections;
* the run loop (solver.py:338-422, 706-800, 1095-1160, 1395-1513): dt starts from the CFL rule, every
  attempt takes dt = min(dt, t_end - t), a rejected attempt leaves U and t
  and retries with dt_next; after an accepted attempt the solver applies its
  post-step operator: the spectral filter for Fourier Euler 1D/2D/3D
  (solver.py:295-323, 671-691, 1360-1380), filter then clamp then projection
  for 2D MHD (1067-1084);
* the right-hand sides: 1D with artificial viscosity and gravity
  (solver.py:295-299), 2D and 3D with gravity but without artificial
  viscosity (the reference passes None there: solver.py:674-675, 1363-1364),
  2D MHD ideal (1069-1070).  No positivity clamp inside the stages.

Parity pin: tests/golden/adaptive.npz, made by running the reference's own
solvers (tests/golden/make_golden.py, section "adaptive").
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, List, Optional, Tuple

import numpy as np

TABLEAUX = {
    # Bogacki-Shampine 3(2): stages, a (strictly lower), b_high, b_low, embedded order
    "rk23": dict(
        a=[[], [1 / 2], [0.0, 3 / 4], [2 / 9, 1 / 3, 4 / 9]],
        b_high=[2 / 9, 1 / 3, 4 / 9, 0.0],
        b_low=[7 / 24, 1 / 4, 1 / 3, 1 / 8],
        order_low=2,
    ),
    # Dormand-Prince 5(4)
    "rk45": dict(
        a=[[], [1 / 5], [3 / 40, 9 / 40], [44 / 45, -56 / 15, 32 / 9],
           [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
           [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
           [35 / 384, 0.0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]],
        b_high=[35 / 384, 0.0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84, 0.0],
        b_low=[5179 / 57600, 0.0, 7571 / 16695, 393 / 640, -92097 / 339200, 187 / 2100, 1 / 40],
        order_low=4,
    ),
    # the reference's simplified 8-stage table named "rk78" (adaptive.py:250-268)
    "rk78": dict(
        a=[[], [1 / 6], [1 / 12, 1 / 4], [1 / 8, 0.0, 3 / 8], [13 / 72, 0.0, 0.0, 11 / 72],
           [5 / 24, 0.0, 0.0, 0.0, 5 / 24], [1 / 20, 0.0, 0.0, 0.0, 0.0, 1 / 20],
           [1 / 8, 0.0, 0.0, 0.0, 0.0, 0.0, 1 / 8]],
        b_high=[1 / 8, 0.0, 0.0, 0.0, 0.0, 0.0, 1 / 8, 0.0],
        b_low=[1 / 9, 0.0, 0.0, 0.0, 0.0, 0.0, 1 / 9, 1 / 9],
        order_low=7,
    ),
}


@dataclass
class Controller:
    """AdaptiveStepController (adaptive.py:23-81) with the solver's
    adaptive_config defaults (solver.py:182-193)."""

    rtol: float = 1e-6
    atol: float = 1e-8
    safety_factor: float = 0.9
    min_dt_factor: float = 0.1
    max_dt_factor: float = 5.0
    max_rejections: int = 10

    def new_dt(self, dt: float, err: float, scale: float, order: int) -> Tuple[float, bool]:
        tol = self.atol + self.rtol * scale
        accept = err <= tol
        if err > 0:
            dt_opt = dt * (tol / err) ** (1.0 / order) * self.safety_factor
            dt_new = dt * float(np.clip(dt_opt / dt, self.min_dt_factor, self.max_dt_factor))
        else:
            dt_new = dt * self.max_dt_factor
        return dt_new, accept


def embedded_step(rhs: Callable[[np.ndarray], np.ndarray], U: np.ndarray, dt: float, method: str):
    """One embedded RK attempt (adaptive.py:165-187, 216-238, 270-292):
    returns (U_high, U_low, err) with err = max |U_high - U_low|."""
    tab = TABLEAUX[method]
    s = len(tab["b_high"])
    k: List[np.ndarray] = []
    for i in range(s):
        Us = U.copy()
        for j, aij in enumerate(tab["a"][i]):
            Us += dt * aij * k[j]
        k.append(rhs(Us))
    Uh = U.copy()
    Ul = U.copy()
    for i in range(s):
        Uh += dt * tab["b_high"][i] * k[i]
        Ul += dt * tab["b_low"][i] * k[i]
    return Uh, Ul, float(np.max(np.abs(Uh - Ul)))


def run_adaptive(rhs: Callable[[np.ndarray], np.ndarray], post: Callable[[np.ndarray], np.ndarray],
                 U0: np.ndarray, t0: float, t_end: float, dt0: float, method: str,
                 ctrl: Optional[Controller] = None, max_attempts: Optional[int] = None):
    """The reference's run loop with the adaptive stepper.  Returns the final
    state and time, the per-attempt log [(dt, accepted)], the proposed dt for
    the next attempt and the consecutive-rejection count."""
    ctrl = ctrl or Controller()
    order = TABLEAUX[method]["order_low"]
    U = U0.copy()
    t = float(t0)
    dt = float(dt0)
    rej = 0
    log: List[Tuple[float, bool]] = []
    while t < t_end - 1e-12:
        if max_attempts is not None and len(log) >= max_attempts:
            break
        dt = min(dt, t_end - t)
        scale = float(np.max(np.abs(U)))
        Uh, _, err = embedded_step(rhs, U, dt, method)
        dt_next, accept = ctrl.new_dt(dt, err, scale, order)
        if not accept:
            rej += 1
            if rej >= ctrl.max_rejections:
                rej = 0
                accept = True
        else:
            rej = 0
        if accept:
            U = post(Uh)
            t += dt
        log.append((dt, accept))
        dt = dt_next
    return U, t, log, dt, rej


def euler_hooks(solver) -> Tuple[Callable, Callable]:
    """(rhs, post) of an oracle EulerSolver on the adaptive path."""
    if solver.ndim == 1:
        rhs = solver.rhs
    else:
        def rhs(U, _s=solver):
            av, _s.av = _s.av, None
            try:
                return _s.rhs(U)
            finally:
                _s.av = av
    return rhs, solver.box.filt


def mhd_hooks(solver) -> Tuple[Callable, Callable]:
    """(rhs, post) of an oracle MHDSolver2D on the adaptive path."""
    return solver.rhs, (lambda U: solver.project(solver.clamp(solver.box.filt(U))))
