"""Annotation-only stand-in for jaxtyping, used when importing the reference
renderer to generate golden fixtures. `Float[...]`, `Int[...]`, `Bool[...]`
subscript to `typing.Any`."""
import typing


class _Sub:
    def __getitem__(self, item):
        return typing.Any


Float = Int = Bool = Shaped = _Sub()
