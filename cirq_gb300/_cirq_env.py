"""Makes ``import cirq`` work where cirq's plotting/dataframe/async extras are absent.

cirq-core imports ``pandas``, ``duet`` and ``matplotlib`` at module top
(``cirq/_compat.py:35``, ``cirq/work/sampler.py:23``, ``cirq/study/result.py``,
``cirq/vis/*``), although none of them is used by state-vector or
density-matrix simulation.  On machines where those packages are not
installed, ``ensure_cirq()`` registers small placeholder modules for exactly
the missing ones and imports cirq again.  Real packages always win: a
placeholder is only created after a real import has failed.

Placeholders behave as follows:

* every attribute is a distinct empty class, so ``isinstance(x, pd.DataFrame)``
  is simply ``False`` and decorators/annotations evaluate;
* ``duet.sync`` / ``duet.run`` / ``duet.pstarmap_async`` run coroutines with
  ``asyncio`` so ``Sampler.run_batch`` still works;
* calling anything else raises ``ImportError`` naming the missing package.
"""

from __future__ import annotations

import asyncio
import importlib
import importlib.util
import importlib.abc
import importlib.machinery
import os
import sys
import types

_PLACEHOLDER_ROOTS = ("pandas", "duet", "matplotlib", "mpl_toolkits")


class _Missing:
    """Stand-in attribute of a placeholder module."""

    _pkg = "?"

    def __init__(self, *a, **k):
        raise ImportError(f"{self._pkg} is not installed; this cirq feature needs it")


class _PlaceholderModule(types.ModuleType):
    def __init__(self, name: str):
        super().__init__(name)
        self.__path__ = []  # behave like a package so submodule imports resolve
        self.__file__ = f"<placeholder {name}>"
        self._cache: dict[str, object] = {}

    def __getattr__(self, attr: str):
        if attr.startswith("__") and attr.endswith("__"):
            raise AttributeError(attr)
        if attr not in self._cache:
            root = self.__name__.split(".")[0]
            self._cache[attr] = type(attr, (_Missing,), {"_pkg": root})
        return self._cache[attr]


def _duet_module() -> types.ModuleType:
    m = _PlaceholderModule("duet")

    def run(fn, *args, **kwargs):
        return asyncio.run(fn(*args, **kwargs))

    def sync(fn):
        def wrapper(*args, **kwargs):
            return asyncio.run(fn(*args, **kwargs))

        wrapper.__name__ = getattr(fn, "__name__", "sync")
        wrapper.__doc__ = getattr(fn, "__doc__", None)
        return wrapper

    async def pstarmap_async(fn, iterable, limit=None):
        return [await fn(*args) for args in iterable]

    async def pmap_async(fn, iterable, limit=None):
        return [await fn(a) for a in iterable]

    def completed_future(value):
        fut = asyncio.get_event_loop().create_future()
        fut.set_result(value)
        return fut

    m.run = run
    m.sync = sync
    m.pstarmap_async = pstarmap_async
    m.pmap_async = pmap_async
    m.completed_future = completed_future
    m.AwaitableFunc = object
    return m


class _PlaceholderFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def __init__(self, roots):
        self.roots = set(roots)

    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in self.roots:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        if spec.name == "duet":
            return _duet_module()
        return _PlaceholderModule(spec.name)

    def exec_module(self, module):
        return None


def _missing_roots() -> list[str]:
    out = []
    for root in _PLACEHOLDER_ROOTS:
        try:
            importlib.import_module(root)
        except ImportError:
            out.append(root)
    return out


def ensure_cirq(extra_paths: tuple[str, ...] = ()) -> types.ModuleType:
    """Imports and returns ``cirq``, adding placeholders for absent extras.

    ``extra_paths`` (and the ``CIRQ_GB300_CIRQ_PATH`` environment variable,
    ``os.pathsep``-separated) are appended to ``sys.path`` when cirq itself is
    not importable from the current path.
    """
    if "cirq" in sys.modules and hasattr(sys.modules["cirq"], "Simulator"):
        return sys.modules["cirq"]
    paths = list(extra_paths)
    env = os.environ.get("CIRQ_GB300_CIRQ_PATH")
    if env:
        paths.extend(p for p in env.split(os.pathsep) if p)
    if importlib.util.find_spec("cirq") is None:
        for p in paths:
            if os.path.isdir(os.path.join(p, "cirq")) and p not in sys.path:
                sys.path.append(p)
    missing = _missing_roots()
    if missing:
        sys.meta_path.append(_PlaceholderFinder(missing))
    import cirq  # noqa: F401  (raises ModuleNotFoundError if cirq is absent)

    return cirq
