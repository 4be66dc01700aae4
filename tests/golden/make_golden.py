"""Extracts the reference's end-to-end known answer for the finite-temperature sweep from its
own test specification (testsuite/test_vs_ed/test_specs.yaml, entry hubbard_finT_chain: the
4-site Hubbard chain, its exact-diagonalisation energy and the simulation parameters ALF's
test runs) into hubbard_finT_chain.json beside this script.  Run once where the reference
tree is available (the path is the first argument); the tests read only the JSON file.

    python tests/golden/make_golden.py /path/to/ALF
"""
import json
import os
import sys


def parse(path: str) -> dict:
    """The hubbard_finT_chain entry, read as plain text (no YAML library is assumed): the
    scalar keys of the entry and the parameter set of its first simulation, with the
    (dtau, Nwrap) pairs of the later ones."""
    lines = open(path).read().splitlines()
    start = lines.index("hubbard_finT_chain:")
    out, params, variants, cur = {}, {}, [], None
    for ln in lines[start + 1:]:
        if ln and not ln.startswith(" "):
            break  # next top-level entry
        s = ln.strip()
        if s.startswith("ed_energy:"):
            out["ed_energy"] = float(s.split(":", 1)[1])
        elif s.startswith("max_sigma:"):
            out["max_sigma"] = float(s.split(":", 1)[1])
        elif s.startswith("max_delta:"):
            out["max_delta"] = float(s.split(":", 1)[1])
        elif s.startswith("- &hubbard_finT_chain_parameter1"):
            cur = params
        elif s.startswith("- <<: *hubbard_finT_chain_parameter1"):
            cur = {}
            variants.append(cur)
        elif cur is not None and ":" in s and not s.startswith("- "):
            k, v = (x.strip() for x in s.split(":", 1))
            v = v.strip('"')
            if v in ("true", "false"):
                val = v == "true"
            else:
                try:
                    val = int(v)
                except ValueError:
                    try:
                        val = float(v)
                    except ValueError:
                        val = v
            cur[k] = val
    out["parameters"] = params
    out["dtau_nwrap"] = [(params["dtau"], params["Nwrap"])] + [(v["dtau"], v["Nwrap"]) for v in variants]
    out["source"] = "testsuite/test_vs_ed/test_specs.yaml, hubbard_finT_chain"
    return out


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "."
    data = parse(os.path.join(ref, "testsuite", "test_vs_ed", "test_specs.yaml"))
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hubbard_finT_chain.json")
    with open(dst, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")
    print(dst)
