"""The connector that routes a piquasso simulator's permanents to the GB300 engine.

piquasso's simulators do their numerics through a connector object.  The
NumPy connector binds ``permanent`` and ``permanent_laplace`` to the compiled
module ``piquasso._math.permanent`` as instance methods that drop ``self``
(reference: piquasso/_simulators/connectors/numpy_/connector.py:20-23,53-54,
with the wrapper ``instancemethod`` of
piquasso/_simulators/connectors/connector.py:27-31).  The passive simulator's
sampler calls ``state._connector.permanent_laplace`` once per photon step
(piquasso/_simulators/passive/simulation_steps.py:342-348) and the exact
probabilities call ``connector.permanent`` (passive/utils.py:131-138).

:class:`GB300Connector` is that NumPy connector with both methods bound to
:mod:`piquasso_gb300.permanent` instead.  It subclasses ``NumpyConnector``,
so ``PassiveSimulator(d, connector=GB300Connector())`` passes the
simulator's connector check (piquasso/_simulators/simulator.py:36-51: a
built-in connector must be an instance of a supported class), and every other
connector method stays NumPy's.

When piquasso itself is not importable, ``GB300Connector`` is None and
:func:`connector_class` builds the same class over any base given to it.
"""

import importlib

# the module (the package's name ``permanent`` is the function it exports)
_permanent = importlib.import_module(__package__ + ".permanent")


def _bound(name):
    """An instance method that forwards its arguments (without ``self``) to
    ``piquasso_gb300.permanent.<name>``, looked up at call time."""

    def method(self, *args, **kwargs):
        return getattr(_permanent, name)(*args, **kwargs)

    method.__name__ = name
    method.__qualname__ = "GB300Connector." + name
    method.__doc__ = getattr(_permanent, name).__doc__
    return method


class GB300PermanentMethods:
    """The two permanent methods of the connector, as a mixin: placed before a
    connector class in the bases, they override its ``permanent`` and
    ``permanent_laplace``."""

    permanent = _bound("permanent")
    permanent_laplace = _bound("permanent_laplace")


def connector_class(base=None):
    """A connector class whose permanents run on the GB300 engine: ``base``
    (default: piquasso's ``NumpyConnector``) with ``permanent`` and
    ``permanent_laplace`` replaced.  Raises ImportError when no base is given
    and piquasso is not importable."""
    if base is None:
        from piquasso._simulators.connectors.numpy_.connector import NumpyConnector as base
    return type("GB300Connector", (GB300PermanentMethods, base),
                {"__doc__": "%s whose permanents run on the GB300 engine." % base.__name__,
                 "__module__": __name__})


try:
    GB300Connector = connector_class()
except ImportError:  # piquasso is not installed here
    GB300Connector = None
