"""GB300 (sm_103a) implementation of the ExSHalos mock-generation path.

Mirrors the reference's Python API for this path (pyexshalos.mock,
pyexshalos.simulation, pyexshalos.utils and the pyexshalos.lib extensions);
every call runs on the GPU through libexh_gb300.so.
"""
__version__ = "1.0.0"
