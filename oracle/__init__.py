"""CPU oracle (test infrastructure only): NumPy restatement of the reference's MATLAB path."""
from .ofrr_oracle import *  # noqa: F401,F403
