"""Contraction drivers: the abstract :class:`Contraction`, the path-driven
:class:`SimpleContraction` and the tree-executor :class:`GpuContraction`."""

from .abc import Contraction

__all__ = ("Contraction",)
