"""The flat parameter vector of the differentiation helpers, on the host: parameter vectors become
device tables and raw per-table-entry gradients become vector gradients by indexing alone, and both
agree with the dictionary forms (``ParameterVector.apply`` + ``ForceField.tables()``,
``ParameterGradient.from_rows``)."""

import numpy as np
import pytest

from xreac_gb300 import ForceField
from xreac_gb300.calculator import ParameterGradient
from xreac_gb300.differentiation import ParameterVector


@pytest.mark.parametrize("name", ["ffield.reax.HO.2015", "ffield.reax.TiOH.Kim2013", "ffield.reax.CHO.2008"])
def test_vector_tables_equal_the_tables_of_the_modified_force_field(name):
    ff = ForceField.bundled(name)
    vec = ParameterVector(ff)
    base = ff.tables()
    theta0 = vec.values(ff)
    pair, angle = vec.tables(base, theta0[None])
    np.testing.assert_array_equal(pair[0], base["pair"])
    np.testing.assert_array_equal(angle[0], base["angle"])
    rng = np.random.default_rng(0)
    thetas = theta0 * (1 + rng.uniform(-0.05, 0.05, (3, len(theta0))))
    pair, angle = vec.tables(base, thetas)
    for k in range(3):
        want = vec.apply(ff, thetas[k]).tables()
        np.testing.assert_array_equal(pair[k], want["pair"])
        np.testing.assert_array_equal(angle[k], want["angle"])
        np.testing.assert_array_equal(vec.values(vec.apply(ff, thetas[k])), thetas[k])


@pytest.mark.parametrize("name", ["ffield.reax.HO.2015", "ffield.reax.TiOH.Kim2013"])
def test_gradient_rows_equal_the_dictionary_gradient(name):
    ff = ForceField.bundled(name)
    vec = ParameterVector(ff)
    T = len(ff.elements)
    rows = ff.angle_row_keys()
    rng = np.random.default_rng(1)
    pair = rng.normal(size=(2, T * T, 28))
    angle = rng.normal(size=(2, len(rows), 7))
    got = vec.gradient_rows(pair, angle)
    for k in range(2):
        want = vec.gradient(ParameterGradient.from_rows(ff, pair[k], angle[k], rows))
        np.testing.assert_allclose(got[k], want, rtol=1e-14, atol=1e-14)
