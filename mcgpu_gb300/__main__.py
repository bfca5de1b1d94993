"""``python -m mcgpu_gb300 <input.config|input.state> [options]``: the
reference's ``metrosim`` command line on the GPU (see ``metrosim``)."""
import sys

from .metrosim import main

sys.exit(main())
