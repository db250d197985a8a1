"""`python -m fans_gb300 <input.json> <output.h5> [--precision fp64|mixed]`: the FANS executable."""
import sys

from .run import main

sys.exit(main())
