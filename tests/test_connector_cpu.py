"""CPU tests of the connector binding (piquasso_gb300.connector).

piquasso itself cannot be imported in this environment, so the binding is
checked over a stand-in base class built like the reference's NumPy
connector: methods that drop ``self`` and forward to a module function
(reference: piquasso/_simulators/connectors/connector.py:27-31,
numpy_/connector.py:53-54).  The GB300 connector must override exactly the two
permanent methods, forward every argument (positional and keyword, as the
sampler and the probability code call them) to piquasso_gb300.permanent, and
leave the base's other methods alone.  No GPU call is made: the engine
functions are replaced by recorders.
"""

import numpy as np
import pytest

from piquasso_gb300 import connector


def _instancemethod(func):
    def wrapped(self, *args, **kwargs):
        return func(*args, **kwargs)

    return wrapped


class StandInNumpyConnector:
    """Shaped like piquasso's NumpyConnector for the methods that matter here."""

    permanent = _instancemethod(lambda *a, **k: ("numpy-permanent", a, k))
    permanent_laplace = _instancemethod(lambda *a, **k: ("numpy-laplace", a, k))
    svd = _instancemethod(np.linalg.svd)


@pytest.fixture
def recorded(monkeypatch):
    import importlib

    perm_mod = importlib.import_module("piquasso_gb300.permanent")
    calls = []
    monkeypatch.setattr(perm_mod, "permanent", lambda *a, **k: calls.append(("permanent", a, k)) or 7.0)
    monkeypatch.setattr(perm_mod, "permanent_laplace",
                        lambda *a, **k: calls.append(("permanent_laplace", a, k)) or np.array([1.0]))
    return calls


def test_connector_overrides_the_two_permanent_methods(recorded):
    cls = connector.connector_class(StandInNumpyConnector)
    c = cls()
    assert isinstance(c, StandInNumpyConnector)
    A = np.eye(3)
    # keyword call, as passive/utils.py:134 makes it
    assert c.permanent(A, rows=[1, 1, 1], cols=[1, 1, 1]) == 7.0
    # positional call (output as rows, input as cols), as sampling.py:732-734
    c.permanent_laplace(A, [1, 0, 0], [1, 1, 0])
    assert recorded[0] == ("permanent", (A,), {"rows": [1, 1, 1], "cols": [1, 1, 1]})
    assert recorded[1] == ("permanent_laplace", (A, [1, 0, 0], [1, 1, 0]), {})
    # every other method is the base's
    u, s, vh = c.svd(np.eye(2))
    assert np.allclose(s, [1.0, 1.0])


def test_connector_binds_the_engine_functions():
    import piquasso_gb300

    cls = connector.connector_class(StandInNumpyConnector)
    assert cls.permanent.__doc__ == piquasso_gb300.permanent.__doc__
    assert cls.permanent_laplace.__doc__ == piquasso_gb300.permanent_laplace.__doc__
    assert cls.__name__ == "GB300Connector"


def test_connector_over_the_reference_when_importable():
    """Where piquasso is installed, GB300Connector subclasses its
    NumpyConnector; here it is None (piquasso is not importable)."""
    try:
        from piquasso._simulators.connectors.numpy_.connector import NumpyConnector
    except ImportError:
        assert connector.GB300Connector is None
        with pytest.raises(ImportError):
            connector.connector_class()
        return
    assert issubclass(connector.GB300Connector, NumpyConnector)
