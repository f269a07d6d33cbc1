"""Extract the positional parameter lists of the reference functions that the
Julia drop-in shim (npbapps.jl_gb300/julia/NPBAppsGPUShim.jl) overrides.

Generates tests/golden/reference_signatures.json from the `function` headers
of (NPBApps.jl):
  src/BT/adi.jl:5-80            adi        (BT-MZ)
  src/SP/adi.jl:6-104           adi        (SP-MZ)
  src/BT/exchange_qbc.jl:1-26   exch_qbc   (BT-MZ)
  src/SP/exchange_qbc.jl:1-26   exch_qbc   (SP-MZ)
  src/LU/ssor.jl:9-50           ssor       (LU-MZ)
  src/LU/exchange_qbc.jl:17     exch_qbc   (LU-MZ)
Each entry is the list of parameter names in call order, with type
annotations and defaults dropped (`_::Val{ncells}` becomes `_`).
Run once where the reference tree is present:
  python tests/golden/make_reference_signatures.py /path/to/NPBApps.jl
The JSON it writes is committed; nothing at test time reads the reference.
"""
import json
import re
import sys
from pathlib import Path

FUNCTIONS = {
    "BT.adi": ("src/BT/adi.jl", "adi"),
    "SP.adi": ("src/SP/adi.jl", "adi"),
    "BT.exch_qbc": ("src/BT/exchange_qbc.jl", "exch_qbc"),
    "SP.exch_qbc": ("src/SP/exchange_qbc.jl", "exch_qbc"),
    "LU.ssor": ("src/LU/ssor.jl", "ssor"),
    "LU.exch_qbc": ("src/LU/exchange_qbc.jl", "exch_qbc"),
}


def strip_comments(text):
    return "\n".join(line.split("#", 1)[0] for line in text.splitlines())


def parameters(path, name):
    """Parameter names of the first `function name(` in path, and its line."""
    raw = Path(path).read_text()
    m = re.search(r"^[ \t]*function[ \t]+" + re.escape(name) + r"[ \t]*\(", raw, re.M)
    if not m:
        raise SystemExit(f"{path}: no function {name}")
    line = raw.count("\n", 0, m.start()) + 1
    text = strip_comments(raw[m.end():])
    depth, args, cur = 1, [], ""
    for ch in text:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
            if depth == 0:
                break
        if ch == "," and depth == 1:
            args.append(cur)
            cur = ""
        else:
            cur += ch
    args.append(cur)
    names = []
    for a in args:
        a = a.strip()
        if not a:
            continue
        a = a.split("=", 1)[0].split("::", 1)[0].strip()
        names.append(a)
    return names, line


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_signatures.py <NPBApps.jl source tree>")
    root = Path(sys.argv[1])
    data = {"source": "NPBApps.jl function headers; parameter names in positional order"}
    for key, (rel, fn) in FUNCTIONS.items():
        names, line = parameters(root / rel, fn)
        data[key] = {"file": f"{rel}:{line}", "params": names}
    dst = Path(__file__).with_name("reference_signatures.json")
    dst.write_text(json.dumps(data, indent=1) + "\n")
    print("wrote", dst, {k: len(v["params"]) for k, v in data.items() if k != "source"})


if __name__ == "__main__":
    main()
