"""Extension-level API, mirroring pyexshalos.lib (pyexshalos/lib/__init__.py:1-4).

`exshalos` and `spectrum` keep the function names and positional argument
orders of the reference's CPython extensions; they call the CUDA library
through its C ABI.
"""
from . import exshalos, spectrum  # noqa: F401
