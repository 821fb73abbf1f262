"""Regenerate models.json in this directory from the Piranha model files.

Run with the Piranha source tree as the first argument (or in the
environment variable PIRANHA_SRC):

    python tests/golden/make_models.py /path/to/piranha

It parses each of Piranha's model files (files/models/*.json) with
piranha_gb300.nets.from_model (which reads the fields as Piranha's
src/util/model.cu does) and writes, per file, either the layer tuples and
the file's batch size / input size / class count, or the reason the file
holds a layer outside this library's layers. Nothing under tests/ reads the
reference tree at test time; only this generator does.
"""
from __future__ import annotations

import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from piranha_gb300 import nets  # noqa: E402


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PIRANHA_SRC", "")
    if not ref or not os.path.isdir(os.path.join(ref, "files", "models")):
        sys.exit("usage: make_models.py <Piranha source tree> (or set PIRANHA_SRC)")
    out = {}
    for path in sorted(glob.glob(os.path.join(ref, "files", "models", "*.json"))):
        name = os.path.basename(path)[:-5]
        try:
            layers, meta = nets.load_model(path)
            out[name] = {"layers": [list(L) for L in layers], "meta": meta}
        except json.JSONDecodeError as e:
            out[name] = {"invalid_json": str(e)}
        except ValueError as e:
            out[name] = {"unsupported": str(e)}
    with open(os.path.join(HERE, "models.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
