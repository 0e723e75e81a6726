"""lair's ``InvalidInput`` error (src/lib.rs:23-30) as Python exceptions."""
from __future__ import annotations


class InvalidInput(ValueError):
    """An invalid function argument.  ``InvalidInput.Shape`` and
    ``InvalidInput.Value`` are the two variants; their ``str`` matches lair's
    ``Display`` ("shape error: ..." / "value error: ...")."""

    kind = "invalid input"

    def __init__(self, message: str):
        super().__init__(f"{self.kind}: {message}")
        self.message = message


class _Shape(InvalidInput):
    kind = "shape error"


class _Value(InvalidInput):
    kind = "value error"


InvalidInput.Shape = _Shape
InvalidInput.Value = _Value
