"""Build recipe for the CPU oracles (test infrastructure only).

* ``oracle/libko_oracle.so``  -- the plain-C FP64 restatement (ko_oracle.c),
  built with -ffp-contract=off and OpenMP.
* ``oracle/_ref/libko_ref64.so`` / ``libko_ref32.so`` -- the reference's own
  src/Kobayashi.cpp compiled unmodified against ref_shim/Win32App.h through
  ref_harness.cpp (FP64 with ``float`` -> ``double``, and FP32 as shipped).

The reference sources are read from the reference checkout named by the
``KO_REFERENCE_DIR`` environment variable and staged, re-encoded from
the file's CP949 to UTF-8 (only the Korean button captions change bytes), into
``oracle/_ref/src/``; that folder is git-ignored and travels with the working
tree so a machine without the checkout can rebuild the same libraries from the
staged copy.  Nothing here runs the reference's own build system.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("KO_REFERENCE_DIR", "")
REF_OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(REF_OUT, "src")
CC = os.environ.get("CC", "gcc")
CXX = os.environ.get("CXX", "g++")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(out, srcs):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs)


def _link_atomic(cmd_without_output, out):
    """compile to a temporary file and rename it over `out`: a process that has the old library
    mapped keeps its copy intact"""
    tmp = out + ".tmp%d" % os.getpid()
    try:
        _run(cmd_without_output + ["-o", tmp])
        os.replace(tmp, out)
    finally:
        if os.path.exists(tmp):
            os.remove(tmp)


def build_port(force=False):
    src = os.path.join(HERE, "ko_oracle.c")
    hdr = [os.path.join(HERE, "..", "crystalgrowth_gb300", "csrc", f) for f in ("kg_math.h", "kg_math_tables.h")]
    out = os.path.join(HERE, "libko_oracle.so")
    if force or not _newer(out, [src] + hdr):
        _link_atomic([CC, "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", src, "-lm"], out)
    return out


def stage_reference():
    """Copy src/Kobayashi.{h,cpp} from the reference checkout named by KO_REFERENCE_DIR into _ref/src.
    Without KO_REFERENCE_DIR the copy staged earlier is used; without either, nothing is built."""
    srcdir = os.path.join(REF_DIR, "src") if REF_DIR else ""
    if not srcdir or not os.path.isfile(os.path.join(srcdir, "Kobayashi.cpp")):
        if REF_DIR:
            raise FileNotFoundError("KO_REFERENCE_DIR=%s holds no src/Kobayashi.cpp" % REF_DIR)
        return os.path.isfile(os.path.join(STAGE, "Kobayashi.cpp"))
    os.makedirs(STAGE, exist_ok=True)
    for name in ("Kobayashi.cpp", "Kobayashi.h"):
        raw = open(os.path.join(srcdir, name), "rb").read()
        text = raw.decode("cp949")
        with open(os.path.join(STAGE, name), "w", encoding="utf-8") as f:
            f.write(text)
    return True


def build_reference(force=False):
    """Returns the list of built libraries, or [] when no reference source is available."""
    if not stage_reference():
        sys.stderr.write("build_oracle: no reference source (KO_REFERENCE_DIR is unset and nothing is staged in %s); "
                         "only the C restatement is built\n" % STAGE)
        return []
    harness = os.path.join(HERE, "ref_harness.cpp")
    shim = os.path.join(HERE, "ref_shim", "Win32App.h")
    deps = [harness, shim, os.path.join(STAGE, "Kobayashi.cpp"), os.path.join(STAGE, "Kobayashi.h")]
    outs = []
    for tag, defs in (("64", ["-DKO_REF_FP64"]), ("32", [])):
        out = os.path.join(REF_OUT, "libko_ref%s.so" % tag)
        if force or not _newer(out, deps):
            _link_atomic([CXX, "-O2", "-std=c++14", "-ffp-contract=off", "-fPIC", "-shared", "-fvisibility=hidden",
                          "-w", *defs, "-I", os.path.join(HERE, "ref_shim"), "-I", STAGE, harness], out)
        outs.append(out)
    return outs


def build(force=False):
    port = build_port(force)
    refs = build_reference(force)
    return [port] + refs


if __name__ == "__main__":
    for p in build(force="--force" in sys.argv):
        print(p)
