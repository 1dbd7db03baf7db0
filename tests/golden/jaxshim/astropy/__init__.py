"""astropy stand-in: enough for the reference's modules to import (units are unused on the path)."""
from . import units, constants  # noqa: F401
