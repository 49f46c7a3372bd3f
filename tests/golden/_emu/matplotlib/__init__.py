"""Empty stand-in so the reference's post-processing module imports (fixture generation only)."""
from . import pyplot  # noqa: F401
