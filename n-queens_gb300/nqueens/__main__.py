"""python -m nqueens: the reference's per-N table on the GB300 engine (see cli.py)."""
import sys

from .cli import main

sys.exit(main())
