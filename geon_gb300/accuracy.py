"""Class accuracy of a trace against the FP64 path, with every disagreement
settled by an independent FP64 integration (the arbiter).

The FP64 path reproduces the reference (geodesic.rs:62-117 with RK4 at a fixed
step), including its numerical accidents: a step that straddles r = 2M, or one
that passes close to the polar axis of the (theta, phi) chart, evaluates the
Christoffel symbols where they blow up, and the ray is flung to r ~ 1e30 or
overflows (the reference then reports it Escaped or Diverged,
schwarzschild.rs:109-121, geodesic.rs:89-100). Where another trace (the mixed
path, the fast FP64 mode) assigns a ray a different class, the ray is traced
again in FP64 with 16 RK4 sub-steps per step (Schwarzschild rays with the
planar step of GEON_FP64_FAST, the others with the FP64 parity stepper).
Termination is tested at every
sub-step, so a ray that reaches the capture radius between two of the
reference's tests is captured there; the step cap is the reference's (a ray
escapes only if it does so by the reference's last test, at step
max_steps - 1). Rays of the spherically symmetric metrics (Schwarzschild,
Morris-Thorne) are traced in the frame of their own orbit plane (an exact
rotation of the sphere, an isometry of these metrics), whose equator is far
from the chart's polar axis. The arbiter's class decides which side is right.
"""
import numpy as np

from .geodesic import trace
from .metric import MORRIS_THORNE, SCHWARZSCHILD

SUBSTEPS = 16


def orbit_frame_states(y):
    """Each state (n, 8) of a spherically symmetric metric in the frame of its
    own orbit plane: e1 the radial direction, e2 the direction of its angular
    motion; theta = pi/2, phi = 0, p^theta = 0 there, t, r and their momenta
    unchanged (FP64)."""
    y = np.asarray(y, dtype=np.float64)
    st, ct = np.sin(y[:, 2]), np.cos(y[:, 2])
    sp, cp = np.sin(y[:, 3]), np.cos(y[:, 3])
    e_th = np.stack([ct * cp, ct * sp, -st], 1)
    e_ph = np.stack([-sp, cp, np.zeros_like(sp)], 1)
    w = y[:, 6:7] * e_th + (y[:, 7] * st)[:, None] * e_ph
    out = y.copy()
    out[:, 2] = np.pi / 2
    out[:, 3] = 0.0
    out[:, 6] = 0.0
    out[:, 7] = np.linalg.norm(w, axis=1)
    return out


def clean_escapes(metric, result):
    """Rays that Escaped at the escape radius with a final state on the null
    cone: a real escape, not a ray flung off its geodesic by a step the fixed
    step cannot resolve (those end at r ~ 1e30 or far off the cone, and their
    final state carries no direction). Escape radius: Schwarzschild its
    escape_radius * M, Morris-Thorne |l| = 1000, the Cartesian metrics r = 1000
    (schwarzschild.rs:116, morris_thorne.rs:38-48, minkowski.rs:32-39,
    alcubierre.rs:65-75); a step goes at most a few percent past it."""
    term = np.asarray(result.termination)
    y = np.asarray(result.final_state)
    resid = np.asarray(result.null_residual)
    if metric.kind == SCHWARZSCHILD:
        r, r_esc = y[:, 1], metric.escape_radius * metric.mass
    elif metric.kind == MORRIS_THORNE:
        r, r_esc = np.abs(y[:, 1]), 1000.0
    else:
        r, r_esc = np.linalg.norm(y[:, 1:4], axis=1), 1000.0
    with np.errstate(over="ignore", invalid="ignore"):
        on_cone = resid <= 1e-6 * np.maximum(1.0, y[:, 4] ** 2)
        return (term == 2) & (r <= 1.1 * r_esc) & on_cone


def arbiter_classes(metric, y0, step, max_steps):
    """Termination of each ray of y0 by the arbiter (FP64, step/16, tests at
    every sub-step, the reference's cap)."""
    y0 = np.asarray(y0, dtype=np.float64).reshape(-1, 8)
    if len(y0) == 0:
        return np.zeros(0, dtype=np.int32)
    if metric.kind in (SCHWARZSCHILD, MORRIS_THORNE):
        y0 = orbit_frame_states(y0)
    cap = SUBSTEPS * (int(max_steps) - 1) + 1 if max_steps > 0 else 0
    # Schwarzschild rays on their plane take the planar FP64 step of
    # GEON_FP64_FAST (same RK4 and tests, fused arithmetic, no trigonometry);
    # the other metrics the FP64 parity stepper
    prec = "fp64fast" if metric.kind == SCHWARZSCHILD else "fp64"
    return trace(metric, y0, step / SUBSTEPS, cap, precision=prec).termination


def class_report(metric, y0, step, max_steps, term, term_fp64, check_agreeing=256, seed=0):
    """Compare the classes `term` of a trace with the FP64 path's `term_fp64` on
    the rays y0. Every disagreement is traced by the arbiter; so is a uniform
    sample of `check_agreeing` rays on which the two agree (to catch rays both
    get wrong). Returns counts and fractions over all rays."""
    term = np.asarray(term)
    term_fp64 = np.asarray(term_fp64)
    n = len(term)
    dis = np.flatnonzero(term != term_fp64)
    arb = arbiter_classes(metric, np.asarray(y0)[dis], step, max_steps)
    agree = np.flatnonzero(term == term_fp64)
    rng = np.random.default_rng(seed)
    chk = rng.choice(agree, size=min(check_agreeing, len(agree)), replace=False) if len(agree) else agree
    arb_chk = arbiter_classes(metric, np.asarray(y0)[chk], step, max_steps)
    wrong = int(np.sum(arb != term[dis]))
    return {
        "rays": int(n),
        "raw_mismatch": float(len(dis) / max(n, 1)),
        "disagreements": int(len(dis)),
        "disagreements_arbiter_sides_with_fp64": int(np.sum(arb == term_fp64[dis])),
        "disagreements_arbiter_sides_with_trace": int(np.sum(arb == term[dis])),
        "mismatch_vs_arbiter": float(wrong / max(n, 1)),
        "agreeing_rays_checked": int(len(chk)),
        "agreeing_rays_arbiter_differs": int(np.sum(arb_chk != term[chk])),
        "arbiter": f"FP64 RK4 at step/{SUBSTEPS}, termination tested every sub-step, the reference's cap"
                   + (" (planar fast-FP64 step)" if metric.kind == SCHWARZSCHILD else "")
                   + (", orbit-plane frame" if metric.kind in (SCHWARZSCHILD, MORRIS_THORNE) else ""),
    }
