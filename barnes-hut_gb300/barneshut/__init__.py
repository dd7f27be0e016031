"""GB300-native drop-in for python-bh's ``barneshut`` package.

Same entry point (``BarnesHut(ini)``, python-bh/barneshut/barneshut.py:4-32),
same config keys and step interface (implementations/base.py:34-258); the
``gb300`` implementation runs every phase on one GPU through libbh_gb300.so.
"""
from .barneshut import BarnesHut

__all__ = ["BarnesHut"]
