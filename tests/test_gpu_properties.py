"""The reference's property tests of the split-form RHS (tests/properties.py)
on the CUDA library, in both numerics variants."""

import pytest

import properties as P
from dgcom_gb300 import abi
from dgcom_gb300.device import SWEPhysics2D

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("prop", P.ALL, ids=lambda f: f.__name__)
def test_reference_property_tests_on_the_device(prop, numerics):
    def make(form):
        form.numerics = numerics
        return SWEPhysics2D(form, 0)
    prop(make)
