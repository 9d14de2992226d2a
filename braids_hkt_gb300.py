"""Import shim for the ``braids-hkt_gb300/`` package directory.

The directory name carries a hyphen, which Python's import statement cannot
spell, so this module stands in for it: it points its package search path at
that directory and runs the package's ``__init__``. ``import braids_hkt_gb300``
and ``from braids_hkt_gb300.mesh import ...`` then work from the repository
root.
"""
import os as _os

__path__ = [_os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "braids-hkt_gb300")]

with open(_os.path.join(__path__[0], "__init__.py"), "rb") as _f:
    exec(compile(_f.read(), _os.path.join(__path__[0], "__init__.py"), "exec"))
