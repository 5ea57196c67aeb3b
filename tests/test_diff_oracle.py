"""CPU checks of the FP64 adjoint of the differentiable shading model
(oracle/diffrender.py) against central finite differences (h = 1e-3) of the
same frozen-coverage L2 loss.

The differences are taken with the model's discrete choices frozen at the
unperturbed parameters -- coverage (the visible triangle per pixel), each
uv's repeat offset and its bilinear texel cell -- which is the smooth
function the adjoint differentiates; without that, uvs that cross a texel
boundary under the step add kink error of a few percent.

Tolerances (norm-wise relative error over the sampled parameters): the loss
is quadratic in colours and texels, so central differences are exact there up
to rounding: 1e-6. Positions and uvs enter non-linearly (perspective-correct
barycentrics, 1/area), so h = 1e-3 carries an O(h^2) truncation error, largest
for the sliver triangles at the sphere's poles: 2e-2; the Richardson
combination of h and h/2 cancels the h^2 term: 1e-5."""
import numpy as np
import pytest

from oracle import diffrender as D

import diff_cases

H = 1e-3


@pytest.fixture(scope="module")
def case():
    return diff_cases.small_case()


def fd(case, name, index, h=H):
    base = D.Model(case["pos"], case["col"], case["uv"], case["tri"], case["tex"], case["mvp"], case["vis"])

    def loss(delta):
        p = {k: case[k] for k in ("pos", "col", "uv", "tri", "tex", "mvp", "vis", "target")}
        arr = p[name].copy()
        arr.reshape(-1)[index] += delta
        p[name] = arr
        return D.loss_only(p["pos"], p["col"], p["uv"], p["tri"], p["tex"], p["mvp"], p["vis"], p["target"], frozen=base)
    return (loss(h) - loss(-h)) / (2 * h)


def adjoint(case):
    return D.loss_and_grad(case["pos"], case["col"], case["uv"], case["tri"], case["tex"], case["mvp"], case["vis"],
                           case["target"])


def sample(grad, count, seed):
    flat = np.abs(grad.reshape(-1))
    nz = np.nonzero(flat > 1e-3 * flat.max())[0]
    rng = np.random.default_rng(seed)
    return rng.choice(nz, size=min(count, nz.size), replace=False)


def test_case_has_coverage(case):
    assert (case["vis"] > 0).sum() > 800


@pytest.mark.parametrize("name,slot,tol", [("col", 1, 1e-6), ("tex", 3, 1e-6), ("uv", 2, 2e-2), ("pos", 0, 2e-2)])
def test_adjoint_matches_central_differences(case, name, slot, tol):
    _, grads = adjoint(case)
    g = grads[slot]
    idx = sample(g, 24, seed=slot)
    assert idx.size >= 10
    num = np.array([fd(case, name, i) for i in idx])
    ana = g.reshape(-1)[idx]
    err = np.linalg.norm(num - ana) / np.linalg.norm(num)
    assert err <= tol, f"{name}: FD vs adjoint relative error {err:.3e}"


@pytest.mark.parametrize("name,slot", [("uv", 2), ("pos", 0)])
def test_adjoint_matches_richardson_differences(case, name, slot):
    _, grads = adjoint(case)
    g = grads[slot]
    idx = sample(g, 16, seed=10 + slot)
    num = np.array([(4.0 * fd(case, name, i, H / 2) - fd(case, name, i, H)) / 3.0 for i in idx])
    ana = g.reshape(-1)[idx]
    err = np.linalg.norm(num - ana) / np.linalg.norm(num)
    assert err <= 1e-5, f"{name}: Richardson FD vs adjoint relative error {err:.3e}"


def test_image_matches_forward_interpolation(case):
    """At a pixel, the model's barycentrics reproduce the triangle's vertex
    attributes at its vertices' own projections (sanity of the closed form)."""
    m = D.Model(case["pos"], case["col"], case["uv"], case["tri"], case["tex"], case["mvp"], case["vis"])
    assert np.all(np.abs(m.lam.sum(1) - 1.0) < 1e-12)
    assert np.all(m.lam > -0.5)
