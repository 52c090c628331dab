"""GB300-native propagator contractions (CLQCD/contract drop-in).

``libcontract.so`` (built by ``python -m contract_gb300.build``) exports the
reference's ``contract.h`` C ABI plus the ``contract_gb300.h`` extensions;
``pycontract`` binds the drop-in calls, ``api`` the extensions.
"""
from . import _lib  # noqa: F401

LIB_PATH = _lib.LIB_PATH


def load():
    """Load libcontract.so (raises if it is missing) and return the ctypes handle."""
    return _lib.lib()
