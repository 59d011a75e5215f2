from .displacement_elemental import DisplacementElementalGenerator
from .eigenvector import EigenvectorGenerator
from .elemental import ElementalGenerator

__all__ = ["ElementalGenerator", "EigenvectorGenerator", "DisplacementElementalGenerator"]
