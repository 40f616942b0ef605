"""Alignment caller on the device (pi_aligner_*, pi_similarity,
pi_optimize_alignment) vs the FP64 restatement of cpp/app/align.

Value to 1e-5 absolute (it is -log of a ratio of volumes held to 1e-5
relative), gradient to 2e-5 of its largest entry (the adjoint contract),
Gauss-Newton Hessian to 1e-4 of its largest entry (it squares gradients).
The optimiser is held to the oracle optimiser's first Newton direction and
to the similarity it reaches.
"""
import numpy as np
import pytest

from pointint_gb300 import align, geometry as G
from pointint_gb300.kgrid import standard_kgrid
from test_align_host import ellipsoid, as_or

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kg():
    return standard_kgrid(9, 16)


def problem(seed):
    rng = np.random.default_rng(seed)
    g1 = ellipsoid(rng, 2, offset=False)
    Vb, Fb = G.box_mesh([1.6, 1.1, 0.8])
    g2 = G.make_triangle_mesh(Vb @ G.random_rotation(rng).T + 0.2, Fb)
    return rng, g1, g2


@pytest.mark.parametrize("measure", [align.SIM_OCHIAI, align.SIM_JACCARD, align.SIM_DICE])
def test_similarity_matches_oracle(cuda, kg, measure):
    from oracle import align as ora, oracle as orc
    rng, g1, g2 = problem(10 + measure)
    kgrid = (kg.dirs, kg.kmag, kg.w)
    with align.Aligner(g1, g2, kg) as a:
        V1 = a.fixed_volume()
        V1r = orc.volume_matrix([orc.Obj(g1.type, g1.elems)], kgrid)[0][0, 0]
        assert abs(V1 - V1r) <= 1e-5 * V1r
        for k in range(3):
            d = G.affine_dofs(np.eye(3) + 0.1 * rng.normal(size=(3, 3)), 0.3 * rng.normal(size=3))
            r = a.similarity(d, measure, V1r, align.SIM_ALL)
            ref = ora.similarity(as_or(g1), as_or(g2), d, kgrid, measure, V1r, ora.ALL)
            f = a.similarity(d, measure, V1r, align.SIM_FUNC_ONLY)
            gs = np.abs(ref["gradient"]).max()
            hs = np.abs(ref["hessian"]).max()
            print(f"\nmeasure {measure} #{k}: s {r.similarity:.5f} (oracle {ref['similarity']:.5f}), "
                  f"grad {np.abs(r.gradient - ref['gradient']).max() / gs:.2e}, "
                  f"hess {np.abs(r.hessian - ref['hessian']).max() / hs:.2e}")
            assert abs(r.value - ref["value"]) <= 1e-5 and abs(f.value - ref["value"]) <= 1e-5
            assert f.gradient is None and f.hessian is None
            assert np.abs(r.gradient - ref["gradient"]).max() <= 2e-5 * gs
            assert np.abs(r.hessian - ref["hessian"]).max() <= 1e-4 * hs
            assert np.abs(r.hessian - r.hessian.T).max() <= 1e-12 * hs


@pytest.mark.parametrize("measure", [align.SIM_DICE, align.SIM_OCHIAI])
def test_optimizer_matches_oracle(cuda, kg, measure):
    """From the warm start of a box against an ellipsoid: the first damped
    Newton direction agrees with the oracle's, and ten iterations raise the
    similarity to within 1e-4 of the oracle optimiser's."""
    from oracle import align as ora
    _, g1, g2 = problem(3)
    kgrid = (kg.dirs, kg.kmag, kg.w)
    d0 = align.compute_warm_start(g1, g2)
    np.testing.assert_allclose(d0, ora.compute_warm_start(as_or(g1), as_or(g2)), atol=1e-9)
    with align.Aligner(g1, g2, kg) as a:
        V1 = a.fixed_volume()
        s0 = a.similarity(d0, measure, V1, align.SIM_FUNC_ONLY).similarity
        one = a.optimize(d0, measure, V1, tolerance=1e-12, max_iterations=1)
        st = a.optimize(d0, measure, V1, tolerance=1e-6, max_iterations=10)
    ref1 = ora.optimize_alignment(as_or(g1), as_or(g2), d0, kgrid, measure, V1, 1e-12, 1, first_step_only=True)
    ref = ora.optimize_alignment(as_or(g1), as_or(g2), d0, kgrid, measure, V1, 1e-6, 10)
    delta = one.dofs - d0  # alpha * delta of the first step
    print(f"\nmeasure {measure}: s {s0:.5f} -> {st.similarity:.5f} (oracle {ref['similarity']:.5f}), "
          f"{st.steps} steps, {st.evaluations} evaluations, status '{st.status}'")
    dr = ref1["first_delta"]
    cosang = delta @ dr / (np.linalg.norm(delta) * np.linalg.norm(dr))
    assert cosang > 1 - 1e-4
    assert st.similarity >= s0
    assert abs(st.similarity - ref["similarity"]) <= 1e-4
    assert st.status in ("Converged (gradient norm < tolerance)", "Reached max iterations")


def test_reference_signature_entry_points(cuda, kg):
    """compute_similarity / optimize_alignment with the reference's argument order."""
    _, g1, g2 = problem(5)
    with align.Aligner(g1, g2, kg) as a:
        V1 = a.fixed_volume()
        want = a.similarity(align.IDENTITY, align.SIM_JACCARD, V1, align.SIM_FUNC_GRAD)
    got = align.compute_similarity(g1, g2, align.IDENTITY, kg, align.SIM_JACCARD, V1, align.SIM_FUNC_GRAD)
    assert got.value == want.value and np.array_equal(got.gradient, want.gradient)
    st = align.optimize_alignment(g1, g2, align.IDENTITY, kg, "jaccard", V1, 1e-6, 2, 0.1)
    assert st.iteration <= 1 and st.dofs.shape == (12,)
