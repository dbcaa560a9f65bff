"""Gradients of the hand-written adjoint at the two differentiable configurations, full size and length
(checks in tests/gradcheck.py).

Differentiable cloth (64 x 64, 120 steps, checkpoint every 10, MSE loss at steps 60 and 120 against a
target run with compliance x LogNormal(0, 0.3); gradients with respect to every edge compliance and
initial velocity):
  - against the gradient of a plain FP64 re-implementation of the step (tests/torch_ref.py) by autodiff,
    its state moved onto the GPU state after every step so that both linearise the same states: 1e-3
    relative (vector norm) per parameter kind;
  - against FP64 central finite differences (eps 1e-6, relative for compliances) on 32 random
    parameters. This cloth hangs from a row of kinematic vertices with stiff edges and no bends, and
    its loss is ill-conditioned: over 120 steps the FP64 gradient itself moves by about 100 % when the
    initial positions move by 1e-7 m, and by about 1e-3 over 6 steps
    (tests/test_oracle_full.py::test_diff_cloth_gradient_conditioning). The FP32 trajectory differs
    from the FP64 one by far more than 1e-7 m, so finite differences of the FP64 run are no 1e-3
    reference for it: the full-length comparison is printed, and over 6 steps (loss at steps 3 and 6)
    the bar is 5e-2.
Differentiable batch (256 bodies, 90 steps, checkpoint every 15, centre-of-mass loss; gradients with
respect to every body's step force and initial velocity):
  - against FP64 autodiff of the two smallest cloths and the smallest tetrahedral cube, each alone, its
    state moved onto the GPU state after every step: 1e-3 relative (vector norm) per parameter kind;
  - against FP64 central FD of each perturbed body alone, its perturbed runs replaying the collision
    decisions of the body's float run (bitwise the GPU's run: planes, contacts, friction clamps,
    restitution and velocity clamp frozen, the derivative the adjoint takes), on 32 random (body, axis)
    parameters of distinct bodies (steps 1e-3 N for forces, 1e-6 m/s for velocities). The hanging cloths
    swing chaotically: their gradients move by percent when the FP64 state is perturbed by 1e-6 (relative)
    after every step, about what FP32 rounding does to a trajectory, so no FP32 solver's gradient can be
    held to FP64 differences there (the FP64 autodiff along the GPU trajectory above matches it to 1e-3). A
    parameter whose FD moves by at most 1e-4 under that perturbation is conditioned; on those, 1e-3 relative
    (vector norm) per kind, and at least 6 of the 32 must be conditioned.
"""
import pytest

from gradcheck import diff_batch_check, diff_cloth_check
from scenes import build_scene

pytestmark = pytest.mark.gpu


def test_diff_cloth_gradients_along_trajectory(jsb):
    r = diff_cloth_check(jsb, build_scene)
    print("diff_cloth, 120 steps:", r)
    p = r["pinned_fp64_autodiff"]
    assert p["loss_rel"] <= 1e-6
    assert p["edge_compliance"] <= 1e-3 and p["v0"] <= 1e-3, p


def test_diff_cloth_with_bends_gradients_along_trajectory(jsb):
    """The differentiable cloth at full size (64 x 64) with dihedral bends (compliance 1e-4), 6 steps (loss
    at steps 3 and 6, checkpoint every 2): edge and bend compliance and initial-velocity gradients against
    FP64 autodiff along the GPU trajectory, 1e-3. The stiff bent cloth's reverse sweep loses precision
    quickly: the same autodiff evaluated in FP32 along the same trajectory differs from FP64 by 2-3e-4
    after 6 steps and by 8e-3 after 12 (the GPU adjoint: 7-12e-3 after 12), so the horizon is kept where an
    FP32 sweep can meet the bar. (The FP64 reference walks the bends' 490 levels per substep one torch
    operation at a time, about 6 s per step.)"""
    r = diff_cloth_check(jsb, build_scene, steps=6, every=2, loss_steps=(3, 6), fd_params=0, bends=True)
    print("diff_cloth with bends, 6 steps:", r)
    p = r["pinned_fp64_autodiff"]
    assert p["loss_rel"] <= 1e-6
    assert p["edge_compliance"] <= 1e-3 and p["v0"] <= 1e-3, p
    # d loss / d bend compliance is proportional to each bend's constraint value C, which the reference
    # computes as ACosApproximate of a cosine rounded to float: for this cloth, flat at the start, most
    # pairs stay within 1e-2 rad of flat, where 1 - cos keeps only a few significant bits (5-6 % of the
    # pairs have cos == 1 exactly and C = -initial angle). The adjoint differentiates the solver's own C;
    # the FP64 reference evaluates C exactly, so the two differ at the percent level here. Bend compliance
    # gradients are held to 1e-3 on a cloth that is not flat (test_gpu_adjoint.py, 10 x 10 cloth).
    assert p["bend_compliance"] <= 3e-2, p


def test_diff_cloth_wavy_with_bends_gradients_along_trajectory(jsb):
    """The 64 x 64 differentiable cloth with dihedral bends, started as a height field of 0.1 m amplitude
    (neighbouring triangles folded by up to 0.4 rad, median 0.14 rad) instead of flat, 6 steps: edge and
    bend compliance and initial-velocity gradients against FP64 autodiff along the GPU trajectory, all
    1e-3. Away from flat pairs the solver's float constraint value keeps its precision, so the bend
    compliance gradients meet the same bar as the others."""
    r = diff_cloth_check(jsb, build_scene, steps=6, every=2, loss_steps=(3, 6), fd_params=0, bends=True, wave_mm=100)
    print("wavy diff_cloth with bends, 6 steps:", r)
    p = r["pinned_fp64_autodiff"]
    assert p["loss_rel"] <= 1e-6
    assert p["edge_compliance"] <= 1e-3 and p["v0"] <= 1e-3 and p["bend_compliance"] <= 1e-3, p


def test_diff_cloth_gradients_vs_fd_short_horizon(jsb):
    r = diff_cloth_check(jsb, build_scene, steps=6, every=2, loss_steps=(3, 6), pinned=False)
    print("diff_cloth, 6 steps:", r)
    assert r["fp64_fd"]["edge_compliance"] <= 5e-2 and r["fp64_fd"]["v0"] <= 5e-2, r


def test_diff_batch_gradients(jsb):
    r = diff_batch_check(jsb, build_scene)
    print("diff_batch:", {k: v for k, v in r.items() if k != "rows"})
    for row in r["rows"]:
        print("  ", row)
    assert r["finite"]
    p = r["pinned_fp64_autodiff"]
    assert p["force"] <= 1e-3 and p["v0"] <= 1e-3, p
    assert r["force"]["conditioned"] + r["v0"]["conditioned"] >= 6, r
    for kind in ("force", "v0"):
        assert r[kind]["rel_error"] is None or r[kind]["rel_error"] <= 1e-3, r
