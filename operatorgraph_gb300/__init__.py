"""GB300-native derivation engine for PGA shape grammars (package root)."""
from . import grammar  # noqa: F401

__version__ = "0.1.0"
