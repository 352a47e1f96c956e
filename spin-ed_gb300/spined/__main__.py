"""python -m spined input.yaml [--debug]: the YAML-in / HDF5-out entry point
(app/Main.hs), running the hot path on the GPU through libsed."""
import argparse
import logging
import sys

from .app import run


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="spined", description="Exact diagonalization of quantum many-body systems "
                                 "(SpinED's configuration format; GPU eigensolver).")
    ap.add_argument("input_file", help="input yaml file")
    ap.add_argument("--debug", action="store_true", help="enable debug output from the library")
    ap.add_argument("--no-warm-start", action="store_true", help="ignore eigenvectors already in the output file")
    args = ap.parse_args(argv)
    logging.basicConfig(level=logging.INFO, format="[%(levelname)s] %(message)s")
    run(args.input_file, debug=args.debug, warm_start=not args.no_warm_start)
    return 0


if __name__ == "__main__":
    sys.exit(main())
