"""TIFF writer for the tests (the package's own)."""
from rfba_gb300.tiff import write_tiff  # noqa: F401
