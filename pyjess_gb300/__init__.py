"""GB300-native template matching with the API of PyJess.

The classes below keep PyJess's constructors, properties and iteration
semantics; `Jess.query` runs on the GPU through ``libpjg.so``.
"""

from ._jess import Atom, Hit, HitArrays, Jess, Mat4, Molecule, Query, Template, TemplateAtom

__version__ = "0.1.0"

__all__ = ["Atom", "Hit", "HitArrays", "Jess", "Mat4", "Molecule", "Query", "Template", "TemplateAtom"]
