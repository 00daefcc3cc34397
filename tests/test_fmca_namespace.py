"""``fmca_gb300.FMCA``: the reference module's H2 names with its defaults
(total-degree interpolation, minimum cluster size 0, FP64), py/FMCA.cpp:37-40,
209-220, 448-468."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err

import fmca_gb300.FMCA as FMCA


def cloud():
    rng = np.random.default_rng(7)
    return rng.random((3, 4000)) * 2 - 1, rng.random((3, 3000)) * 2 - 1


def test_module_defaults_and_statistics(capsys):
    Pr, Pc = cloud()
    ker = FMCA.CovarianceKernel("EXPONENTIAL", 2.0)
    assert ker.kernelType() == "EXPONENTIAL"
    assert FMCA.CovarianceKernel().kernelType() == "EXPONENTIAL"
    H = FMCA.H2Matrix(ker, Pr, Pc, 3, 0.8)
    assert H._h.info["interpolator"] == 1 and H._h.info["q"] == 20
    assert H._h.info["min_leaf"] == 20  # max(0, q), like H2ClusterTree::init
    O = oracle.OraclePlan(Pr, Pc, p=3, eta=0.8, min_leaf=0, interpolator="total_degree")
    st = H.statistics()
    assert st.shape == (6, 1)
    assert np.array_equal(st.ravel(), O.statistics())
    assert "number of low rank blocks" in capsys.readouterr().out
    with pytest.raises(TypeError):
        FMCA.H2Matrix(ker, Pr, Pc)  # p and eta are required, as in the module


@pytest.mark.gpu
def test_module_action_equals_oracle(cuda_device):
    Pr, Pc = cloud()
    x = np.random.default_rng(8).standard_normal((3000, 3))
    O = oracle.OraclePlan(Pr, Pc, p=3, eta=0.8, min_leaf=0, interpolator="total_degree")
    y_ref, _ = O.action(0, 2.0, x)
    H = FMCA.H2Matrix(FMCA.CovarianceKernel("EXPONENTIAL", 2.0), Pr, Pc, 3, 0.8)
    assert rel_err(H.action(x), y_ref) < 1e-12
