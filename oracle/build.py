"""Build recipe of the C oracle: ``python oracle/build.py``."""

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from oracle import build  # noqa: E402

if __name__ == "__main__":
    print(build())
