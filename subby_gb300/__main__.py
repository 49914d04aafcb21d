"""Command line: ``python -m subby_gb300 [input.json] [-o out.json]
[--indent N] [--validate]`` — the reference's ``python -m subby``
(subby/__main__.py:10-74): a JSON request (file or standard input) run
through the GPU path, the result as JSON (file or standard output);
``--validate`` only parses the request and exits 0 ("Valid.") or 1
("Invalid: <reason>") with the message on standard error."""
from __future__ import annotations

import argparse
import json
import sys


def main(argv=None):
    from .io import load_input, load_json, run, format_output
    ap = argparse.ArgumentParser(prog="subby_gb300",
                                 description="Phylogenetic sufficient statistics of a JSON request, on the GPU.")
    ap.add_argument("input", nargs="?", help="request JSON file (standard input when omitted)")
    ap.add_argument("-o", "--output", help="output JSON file (standard output when omitted)")
    ap.add_argument("--indent", type=int, default=2, help="JSON indentation (default 2)")
    ap.add_argument("--validate", action="store_true", help="check the request without running it")
    a = ap.parse_args(argv)
    data = load_json(a.input) if a.input else json.load(sys.stdin)
    if a.validate:
        try:
            load_input(data)
        except Exception as e:  # noqa: BLE001  (any parse error makes the request invalid)
            print(f"Invalid: {e}", file=sys.stderr)
            sys.exit(1)
        print("Valid.", file=sys.stderr)
        sys.exit(0)
    text = format_output(run(data), indent=a.indent)
    if a.output:
        with open(a.output, "w") as f:
            f.write(text + "\n")
    else:
        print(text)


if __name__ == "__main__":
    main()
