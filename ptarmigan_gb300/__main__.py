"""python -m ptarmigan_gb300 input.yml [output_dir]: runs a ptarmigan
input file on the GPU (see driver.py for the supported keys)."""

import sys

from .driver import run


def main(argv):
    if len(argv) < 2 or argv[1] in ("-h", "--help"):
        print(__doc__)
        return 0 if len(argv) >= 2 else 2
    files = run(argv[1], argv[2] if len(argv) > 2 else "")
    for f in files:
        print("wrote", f)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
