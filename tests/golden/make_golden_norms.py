"""Extract the NPB-MZ verification norms from the reference's verify.jl files.

Generates tests/golden/npb_golden_norms.json from
  src/BT/verify.jl:136-348, src/SP/verify.jl:137-282 and src/LU/verify.jl
  (LU-MZ: itmaxref, xcrref, xceref and the surface integral xciref; class F's
  second block, for itmax 30, is left out) (NPBApps.jl).
Run once where the reference tree is present:
  python tests/golden/make_golden_norms.py /path/to/NPBApps.jl
The JSON it writes is committed; nothing at test time reads the reference.
"""
import json
import re
import sys
from pathlib import Path


def parse(path):
    text = Path(path).read_text()
    out = {}
    cls = None
    niter = None
    dt = None
    block_re = re.compile(r"class\s*==\s*CLASS_([A-Z])")
    for line in text.splitlines():
        code = line.split("#", 1)[0]
        m = block_re.search(code)
        if m:
            cls = m.group(1)
            out.setdefault(cls, {"xcr": [None] * 5, "xce": [None] * 5})
            continue
        if cls is None:
            continue
        m = re.search(r"dtref\s*=\s*([0-9.eE+-]+)", code)
        if m and "dt" not in out[cls]:
            out[cls]["dt"] = float(m.group(1))
        m = re.search(r"(?:niterref|itmaxref)\s*=\s*(\d+)", code)
        if m and "niter" not in out[cls]:
            out[cls]["niter"] = int(m.group(1))
        m = re.search(r"xciref\s*=\s*([0-9.eE+-]+)", code)
        if m and "xci" not in out[cls]:
            out[cls]["xci"] = float(m.group(1))
        m = re.search(r"(xcrref|xceref)\[(\d)\]\s*=\s*([0-9.eE+-]+)", code)
        if m and None in out[cls]["xcr" if m.group(1) == "xcrref" else "xce"]:
            key = "xcr" if m.group(1) == "xcrref" else "xce"
            out[cls][key][int(m.group(2)) - 1] = float(m.group(3))
    return {k: v for k, v in out.items() if None not in v["xcr"] and None not in v["xce"]}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden_norms.py <NPBApps.jl source tree>")
    root = Path(sys.argv[1])
    data = {
        "source": "NPBApps.jl src/BT/verify.jl:136-348, src/SP/verify.jl:137-282, src/LU/verify.jl "
                  "(epsilon 1e-8, verify.jl:113)",
        "BT": parse(root / "src/BT/verify.jl"),
        "SP": parse(root / "src/SP/verify.jl"),
        "LU": parse(root / "src/LU/verify.jl"),
    }
    dst = Path(__file__).with_name("npb_golden_norms.json")
    dst.write_text(json.dumps(data, indent=1) + "\n")
    print("wrote", dst, {k: sorted(v) for k, v in data.items() if k != "source"})


if __name__ == "__main__":
    main()
