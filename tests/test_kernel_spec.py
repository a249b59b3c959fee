"""Kernel-expression parsing: mirrors src/interpreter/parser.f90 and ast.f90."""
import pytest

from fgpu.kernel_spec import (CONSTANT, LINEAR, PERIODIC, PROD, RBF, RBF_CYCLIC, SUM, KernelSpecError,
                              build_kspec, nparams, parse_expression, parse_kspec)

KS = {"k1": {"type": "rbf"}, "k2": {"type": "periodic", "active_dimensions": [3]},
      "k3": {"type": "rbf-cyclic"}, "k4": {"type": "linear", "active_dimensions": [1, 2]}}


def test_single_kernel_defaults_to_all_dims():
    ks, c = build_kspec("k1", KS, 3)
    assert ks == [RBF, 3, 1, 2, 3] and c == []
    assert nparams(ks) == 3


def test_water_product():
    ks, _ = build_kspec("k1*k2", KS, 3)
    assert ks == [RBF, 3, 1, 2, 3, PERIODIC, 1, 3, PROD]
    assert nparams(ks) == 4


def test_precedence_and_associativity():
    # '*' binds tighter than '+'; '+' left-assoc; '*' right-recursive (parser.f90 term)
    assert parse_expression("k1+k2*k3") == ("+", ("var", "k1"), ("*", ("var", "k2"), ("var", "k3")))
    assert parse_expression("k1*k2*k3") == ("*", ("var", "k1"), ("*", ("var", "k2"), ("var", "k3")))
    assert parse_expression("k1+k2+k3") == ("+", ("+", ("var", "k1"), ("var", "k2")), ("var", "k3"))
    assert parse_expression("(k1+k2)*k3") == ("*", ("+", ("var", "k1"), ("var", "k2")), ("var", "k3"))
    assert parse_expression("+k1") == ("var", "k1")


def test_numbers_become_constant_kernels():
    ks, c = build_kspec("k1+0.5", KS, 3)
    assert ks == [RBF, 3, 1, 2, 3, CONSTANT, 0, SUM] and c == [0.5]
    assert nparams(ks) == 4


@pytest.mark.parametrize("expr,where", [("k1+0.5", 3), ("2.5*k1+0.5", 0), ("k2+(1.5*k1)", 1)])
def test_constant_parameters_start_at_their_value(expr, where):
    """A number's constant kernel starts with its value as its parameter, at
    its own place in the parameter vector (leaf order); the engine is not
    touched (a stand-in is passed)."""
    import numpy as np
    from fgpu.gpr import GaussianProcessRegressor
    X = np.random.default_rng(0).normal(size=(5, 3))
    gp = GaussianProcessRegressor(X, X[:, 0], expr, KS, engine=object())
    ks, consts = build_kspec(expr, KS, 3)
    p = gp.get_params()
    assert p.size == nparams(ks)
    assert p[where] == consts[0]
    if len(consts) > 1:
        assert p[-1] == consts[1]
    assert np.count_nonzero(p) == len(consts)


def test_leaf_order_is_parameter_order():
    ks, _ = build_kspec("k4*(k2+k1)", KS, 3)
    leaves = [n for n in parse_kspec(ks) if n[0] == "leaf"]
    assert [l[1] for l in leaves] == [LINEAR, PERIODIC, RBF]
    assert ks[-2:] == [SUM, PROD]


def test_cyclic_type_code():
    ks, _ = build_kspec("k3", KS, 6)
    assert ks[:2] == [RBF_CYCLIC, 6]


@pytest.mark.parametrize("expr", ["k1-k2", "k1/k2", "-k1", "k1+", "(k1", "k9", "k1 $ k2"])
def test_rejected_expressions(expr):
    with pytest.raises(KernelSpecError):
        build_kspec(expr, KS, 3)


def test_active_dim_out_of_range():
    with pytest.raises(KernelSpecError):
        build_kspec("k2", {"k2": {"type": "periodic", "active_dimensions": [4]}}, 3)


@pytest.mark.parametrize("bad", [[RBF], [RBF, 2, 1], [SUM], [RBF, 1, 1, RBF, 1, 1], [99]])
def test_malformed_spec(bad):
    with pytest.raises(KernelSpecError):
        parse_kspec(bad)
