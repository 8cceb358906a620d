"""Import shim: ``import ethersph_gb300`` loads the package directory
``ethersphcpu.jl_gb300/`` (a directory name Python cannot import directly)."""
import importlib.util as _u
import sys as _s
from pathlib import Path as _P

_root = _P(__file__).resolve().parent / "ethersphcpu.jl_gb300"
_spec = _u.spec_from_file_location(__name__, _root / "__init__.py", submodule_search_locations=[str(_root)])
_mod = _u.module_from_spec(_spec)
_s.modules[__name__] = _mod
_spec.loader.exec_module(_mod)
