"""python -m ptilopsis_gb300: the reference's command line (see cli.py)."""
import sys

from .cli import main

sys.exit(main())
