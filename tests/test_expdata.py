"""ExpData: the reference fields this engine does not implement make the
simulation call raise rather than being ignored, and unknown attributes are
refused (host logic, no GPU)."""
import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import robertson_model
from amici_gb300.simulation import _stack_inputs


@pytest.mark.parametrize("field,value", [("fixed_parameters_pre_equilibration", [1.0]),
                                         ("fixed_parameters_presimulation", [1.0]),
                                         ("t_presim", 5.0), ("x0", [1.0, 0.0, 0.0]),
                                         ("sx0", np.zeros(9))])
def test_unsupported_fields_raise(field, value):
    m = ag.Model(robertson_model())
    e = ag.ExpData(ts=np.linspace(0, 1, 3))
    setattr(e, field, value)
    with pytest.raises(NotImplementedError, match=field):
        _stack_inputs(m, [e])


def test_supported_batch_and_unknown_attribute():
    m = ag.Model(robertson_model())
    e = ag.ExpData(ts=np.linspace(0, 1, 3), measurements=np.zeros((3, 3)))
    p, pscale, k, ts, my, sg = _stack_inputs(m, [e, e])
    assert p.shape == (2, 3) and ts.shape == (2, 3) and my.shape == (2, 3, 3) and sg is None
    with pytest.raises(AttributeError):
        e.fixed_parameters_preequilibration = [1.0]  # misspelt: refused instead of ignored
