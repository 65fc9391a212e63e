"""Stand-in for flax.struct / flax.linen sufficient to import jqmc's data classes."""
from . import struct, linen  # noqa: F401
