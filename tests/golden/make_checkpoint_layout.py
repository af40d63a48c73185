"""Extract the checkpoint file layout from the reference's source text.

Writes checkpoint_layout.json beside this script: the dataset names of the
save block of cpp/h_mec_rsf_v9.cpp (the string arrays matrix_names,
matrix_names_plus, vector_names, vector_names_marker, and the order of the
nine values streamed into `temp`), in write order, plus the group names and
the file-name stem.  The reference's source tree is a required argument:

    python tests/golden/make_checkpoint_layout.py <reference source tree>
"""
import json
import os
import re
import sys


def layout(ref_root: str) -> dict:
    src = open(os.path.join(ref_root, "cpp", "h_mec_rsf_v9.cpp")).read()
    save = src[src.index("if (timestep % savestep == 0)"):]

    def names(var):
        m = re.search(r"const string %s\[\d+\] = \{([^}]*)\}" % var, save)
        return re.findall(r'"([^"]+)"', m.group(1))

    vals = re.search(r"temp << ([^;]*);", save).group(1)
    groups = re.findall(r'const string group_\w+ = "(\w+)";', save)
    consts = open(os.path.join(ref_root, "cpp", "constants.hpp")).read()
    nname = re.search(r'const string nname = "([^"]*)"', consts).group(1)
    return {
        "matrix_basic": names("matrix_names"),
        "matrix_staggered": names("matrix_names_plus"),
        "history": names("vector_names"),
        "markers": names("vector_names_marker"),
        "values": [v.strip() for v in vals.split(",")],
        "groups": groups,
        "nname": nname,
    }


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_checkpoint_layout.py <reference source tree>")
    ref = sys.argv[1]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "checkpoint_layout.json")
    with open(out, "w") as f:
        json.dump(layout(ref), f, indent=1)
        f.write("\n")
    print(out)
