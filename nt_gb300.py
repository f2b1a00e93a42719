"""Import shim: exposes the package directory ``neural-tangents_gb300/`` as ``nt_gb300``."""
import importlib.util as _ilu
import os as _os
import sys as _sys

_DIR = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), 'neural-tangents_gb300')
_spec = _ilu.spec_from_file_location('nt_gb300', _os.path.join(_DIR, '__init__.py'),
                                     submodule_search_locations=[_DIR])
_mod = _ilu.module_from_spec(_spec)
_sys.modules['nt_gb300'] = _mod
_spec.loader.exec_module(_mod)
