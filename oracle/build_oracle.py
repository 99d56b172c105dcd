"""Build recipe for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

* ``oracle/_build/liboracle_sampler.so``: this repository's plain-C
  restatement of the reference sampler (``oracle/sampler.c``).
* ``oracle/_ref/bor_stream_kernel.so``: the reference's own sampler
  (``bor_stream_kernel.c``) compiled from its source where it lies, with the
  compile line the reference documents (bor_stream_kernel.c:18-19).  Built only
  when GHOST_REFERENCE_DIR names the reference tree; it is used to check the
  restatement and to run the reference for the golden fixtures.

Both outputs are git-ignored build products.
"""

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_DIR = os.environ.get("GHOST_REFERENCE_DIR", "")


def _cc(src: str, out: str) -> None:
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle sampler")
    tmp = out + ".tmp"
    subprocess.check_call([cc, "-O3", "-shared", "-fPIC", "-o", tmp, src, "-lm"])
    os.replace(tmp, out)


def build(force: bool = False) -> None:
    out = os.path.join(HERE, "_build", "liboracle_sampler.so")
    src = os.path.join(HERE, "sampler.c")
    if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        _cc(src, out)
    ref_src = os.path.join(REFERENCE_DIR, "bor_stream_kernel.c") if REFERENCE_DIR else ""
    if ref_src and os.path.exists(ref_src):
        ref_out = os.path.join(HERE, "_ref", "bor_stream_kernel.so")
        if force or not os.path.exists(ref_out):
            _cc(ref_src, ref_out)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("oracle built")
