"""CPU FP64 oracle of the LM fitting step (test infrastructure only)."""
from .oracle import OracleFitter, format_peaks, fit_frames, load, build  # noqa: F401
