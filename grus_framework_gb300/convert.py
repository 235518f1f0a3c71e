"""Command line: edge list or Matrix Market coordinate file -> Galois .gr.

  python -m grus_framework_gb300.convert IN OUT [--symmetric] [--weighted]

The reference points its users at Galois' graph-convert for this step
(README.md:14-27); this wraps grus_convert_edgelist.
"""
import argparse

from . import build, convert_edgelist


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("input")
    ap.add_argument("output")
    ap.add_argument("--symmetric", action="store_true", help="add reverse edges, one copy per pair")
    ap.add_argument("--weighted", action="store_true", help="keep the third column as uint32 weights")
    args = ap.parse_args(argv)
    build.build()
    convert_edgelist(args.input, args.output, symmetric=args.symmetric, weighted=args.weighted)


if __name__ == "__main__":
    main()
