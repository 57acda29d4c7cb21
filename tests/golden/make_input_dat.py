"""Generate tests/golden/input_default.dat exactly as the reference's run_cuda.pl writes it.

run_cuda.pl also compiles and edits TTSH3D.cu, so it is never run as a whole: this
script takes only its parameter assignments (run_cuda.pl:7-44) and its input.dat
writer (run_cuda.pl:53-87) and runs those lines with perl in a temporary directory.
Requires the reference sources (development container only); the output is committed.
"""
import os
import shutil
import subprocess
import sys
import tempfile

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "oracle"))
from make_ref import REF_DIR  # noqa: E402

REF = os.path.join(REF_DIR, "run_cuda.pl")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "input_default.dat")


def main():
    lines = open(REF).read().split("\n")
    snippet = "\n".join(lines[6:44] + lines[52:87]) + "\n"
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "snippet.pl"), "w") as fh:
            fh.write(snippet)
        subprocess.check_call(["perl", "snippet.pl"], cwd=d)
        shutil.copy(os.path.join(d, "input.dat"), OUT)
    print(OUT)


if __name__ == "__main__":
    sys.exit(main())
