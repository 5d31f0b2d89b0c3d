"""Make ``import libcasm.monte...`` resolve to this package.

Importing this module registers ``libcasm.monte`` and its submodules (``_monte``,
``sampling``, ``events``, ``methods``, ``ising_cpp``, ``ising_cpp.semigrand_canonical``,
``ising_py``, ``ising_py.semigrand_canonical``) in ``sys.modules`` as the corresponding
``casmcode_monte_gb300`` modules, so that code written against libcasm-monte's Python
package runs unchanged.  It can also be given to pytest as a plugin
(``pytest -p casmcode_monte_gb300.libcasm_alias``) to run such code's tests.
"""
import importlib
import sys
import types

SUBMODULES = ("", "._monte", ".sampling", ".events", ".methods", ".ising_cpp", ".ising_cpp.semigrand_canonical",
              ".ising_py", ".ising_py.semigrand_canonical")


def install() -> None:
    pkg = sys.modules.setdefault("libcasm", types.ModuleType("libcasm"))
    if not hasattr(pkg, "__path__"):
        pkg.__path__ = []
    for sub in SUBMODULES:
        sys.modules["libcasm.monte" + sub] = importlib.import_module("casmcode_monte_gb300" + sub)
    pkg.monte = sys.modules["libcasm.monte"]


install()
