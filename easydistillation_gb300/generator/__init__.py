from .elemental import ElementalGenerator
from .eigenvector import EigenvectorGenerator

__all__ = ["ElementalGenerator", "EigenvectorGenerator"]
