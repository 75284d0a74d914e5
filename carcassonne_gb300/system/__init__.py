"""The 2D center-site system (carcassonne.system)."""
from ._2d import System, sideFromCorner

__all__ = ["System", "sideFromCorner"]
