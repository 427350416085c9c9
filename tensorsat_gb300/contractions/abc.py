"""Abstract base class of contractions (``tensorsat/contractions/abc.py:29-97``).

A contraction is planned once for a wiring and a box class, then contracts any flat
diagram with that wiring (the plan-reuse idiom of the reference, e.g. the assignment
search of ``notebooks/02-random-ksat.ipynb`` that contracts 2n diagrams with one plan).
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Any

from ..diagrams import Box, Diagram, Wiring


class Contraction(ABC):
    """Abstract base class for contractions."""

    def __init__(self, box_class: type, wiring: Wiring) -> None:
        if not (isinstance(box_class, type) and issubclass(box_class, Box)):
            raise TypeError("box_class must be a subclass of Box.")
        if not isinstance(wiring, Wiring):
            raise TypeError("wiring must be a Wiring.")
        if not box_class.can_be_contracted():
            raise ValueError("Given box class cannot be contracted.")
        self._box_class = box_class
        self._wiring = wiring

    @property
    def box_class(self) -> type:
        """Box class associated with this contraction."""
        return self._box_class

    @property
    def wiring(self) -> Wiring:
        """The wiring contracted by this contraction."""
        return self._wiring

    def can_contract(self, diagram: Diagram) -> bool:
        """Whether the diagram can be contracted using this contraction."""
        try:
            self.validate(diagram)
            return True
        except ValueError:
            return False

    def validate(self, diagram: Diagram) -> None:
        """Raises ValueError unless every box is an instance of the box class, the wiring
        matches, no slot is open and the diagram is flat (``abc.py:64-89``)."""
        if not isinstance(diagram, Diagram):
            raise TypeError("Expected a Diagram.")
        if not all(issubclass(cls, self._box_class) for cls in diagram.box_classes):
            raise ValueError(
                f"Cannot contract diagram: diagram box class {diagram.box_class} is"
                f" not a subclass of contraction box class {self._box_class}"
            )
        if diagram.wiring != self._wiring:
            raise ValueError("Diagram's wiring must match contraction wiring.")
        if diagram.num_open_slots > 0:
            raise ValueError("Diagram cannot have open slots.")
        if not diagram.is_flat:
            raise ValueError("Diagram must be flat.")

    @abstractmethod
    def contract(self, diagram: Diagram, *args: Any, **kwargs: Any) -> Box:
        """Validates and contracts the given diagram."""
