"""Import shim for the upstream tensorsat sources (fixture generation only).

The upstream package needs Python >= 3.13 (``TypeVar(..., default=...)``) and the
packages ``hashcons``, ``xxhash`` and ``typing_validation``, none of which are present
in the fixture-generation container (Python 3.12).  This module makes the upstream
sources importable *without modifying them*:

1. a ``sys.meta_path`` finder loads ``tensorsat.*`` from the upstream checkout and
   strips the ``default=...`` keyword from ``TypeVar(...)`` calls at source-load time;
2. minimal stand-ins for ``hashcons.InstanceStore``, ``xxhash.xxh64`` and
   ``typing_validation.validate`` are installed in ``sys.modules``;
3. bytecode writing is disabled so no ``__pycache__`` lands in the upstream tree.

Where the sources come from (:func:`reference_root`): the directory named by the
``TENSORSAT_REFERENCE`` environment variable (an upstream checkout, as
``tests/golden/make_golden.py`` needs for the upstream example files), else the
``baseline/_ref`` install of the unmodified upstream package at the repository root (which
travels with the repository to GPU hosts). ``tests/golden/make_golden.py`` and the
reference-side plugin tests use it; nothing under the product package imports it.
"""

from __future__ import annotations

import contextlib
import hashlib
import importlib.abc
import importlib.util
import os
import re
import sys
import types

REPO_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
INSTALLED_ROOT = os.path.join(REPO_ROOT, "baseline", "_ref")


def candidate_roots() -> list[str]:
    """Directories searched for the upstream ``tensorsat`` package, in order."""
    roots = []
    env = os.environ.get("TENSORSAT_REFERENCE")
    if env:
        roots.append(env)
    roots.append(INSTALLED_ROOT)
    return roots


def reference_root() -> str | None:
    """The first candidate directory that holds ``tensorsat/``, or None."""
    for root in candidate_roots():
        if os.path.isdir(os.path.join(root, "tensorsat")):
            return root
    return None


REFERENCE_ROOT = reference_root() or INSTALLED_ROOT

_TYPEVAR_DEFAULT = re.compile(r"(TypeVar\([^()]*?),\s*default\s*=\s*[A-Za-z_][\w\.]*\s*\)")


def _install_stubs() -> None:
    if "hashcons" not in sys.modules:
        hashcons = types.ModuleType("hashcons")

        class InstanceStore:
            """Hash-consing store: one instance per (class, key)."""

            def __init__(self) -> None:
                self._instances: dict = {}
                self._pending: list = []

            @contextlib.contextmanager
            def instance(self, cls, key):
                full_key = (cls, key)
                existing = self._instances.get(full_key)
                self._pending.append(full_key)
                try:
                    yield existing
                finally:
                    self._pending.pop()

            def register(self, obj) -> None:
                self._instances[self._pending[-1]] = obj

        hashcons.InstanceStore = InstanceStore
        sys.modules["hashcons"] = hashcons
    if "xxhash" not in sys.modules:
        xxhash = types.ModuleType("xxhash")

        class _H:
            def __init__(self, data) -> None:
                self._d = hashlib.blake2b(bytes(data), digest_size=8).digest()

            def intdigest(self) -> int:
                return int.from_bytes(self._d, "little")

        xxhash.xxh64 = _H
        sys.modules["xxhash"] = xxhash
    if "typing_validation" not in sys.modules:
        tv = types.ModuleType("typing_validation")
        tv.validate = lambda *a, **k: True
        sys.modules["typing_validation"] = tv


class _Loader(importlib.abc.SourceLoader):
    def __init__(self, path: str) -> None:
        self._path = path

    def get_filename(self, fullname: str) -> str:
        return self._path

    def get_data(self, path: str) -> bytes:
        with open(path, "rb") as f:
            src = f.read().decode()
        if path.endswith(".py"):
            src = _TYPEVAR_DEFAULT.sub(r"\1)", src)
        return src.encode()


class _Finder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path=None, target=None):
        if fullname != "tensorsat" and not fullname.startswith("tensorsat."):
            return None
        rel = fullname.split(".")
        base = os.path.join(REFERENCE_ROOT, *rel)
        if os.path.isdir(base):
            init = os.path.join(base, "__init__.py")
            return importlib.util.spec_from_file_location(
                fullname, init, loader=_Loader(init), submodule_search_locations=[base]
            )
        if os.path.isfile(base + ".py"):
            return importlib.util.spec_from_file_location(
                fullname, base + ".py", loader=_Loader(base + ".py")
            )
        return None


def install() -> None:
    """Makes ``import tensorsat`` load the upstream sources (idempotent)."""
    sys.dont_write_bytecode = True
    _install_stubs()
    if not any(isinstance(f, _Finder) for f in sys.meta_path):
        sys.meta_path.insert(0, _Finder())


def available() -> bool:
    return reference_root() is not None
