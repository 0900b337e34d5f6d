"""GB300 (sm_103a) device adapter for the Dax uniform-grid isosurface,
threshold and cell-gradient path.

The compute lives in ``lib/libdax_gb300.so`` (C ABI: ``include/dax_gb300.h``);
``cont`` mirrors the ``dax::cont`` dispatchers over it, ``capi`` is the raw
binding, ``synthetic`` generates the seeded benchmark fields.
"""
from . import capi  # noqa: F401

__version__ = "0.1.0"

