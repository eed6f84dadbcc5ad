"""Build recipe for oracle/_ref -- TEST INFRASTRUCTURE ONLY.

Runs the reference's own C loop-nest emitter (``generate_cfunction`` in
trunk/generator2.py:48-130 for rank 4 and trunk/generator6.py:61-134 for
rank 6) from the reference checkout, writes the emitted C into
``oracle/_ref/`` (git-ignored, never committed) and compiles it with
``gcc -O3 -fopenmp -ffp-contract=off`` into ``oracle/_ref/libref_nests.so``.

The emitted text is used verbatim except for one documented patch applied to
the generated artefact (not to any reference source): the emitters declare
``const int f = *factor;`` and ``const int g = *acc_factor;``
(trunk/generator2.py:64-65, trunk/generator6.py:83-84), which truncates
non-integer factors such as 0.5 to 0.  The patch turns both into
``const double``, so the nests compute what their Fortran twins compute.

What is generated:
  * rank 4: all 24 permutations x all 24 loop orders, OpenMP form -- the
    reference's full brute-force search space (trunk/generator2.py:446-629).
  * rank 6: all 720 permutations with the natural loop order (enough for
    parity: any loop order writes every element once), plus, for the 55
    CCSD(T) permutations of trunk/generator6.py:15-17, four loop orders whose
    innermost pair is {6, p6} (a reduced tuning space: the full 720x720 search
    takes hours to compile).

When the reference checkout is absent (as on a machine that only received the
repository copy), ``build()`` compiles whatever generated C is already present
in ``oracle/_ref``.
"""
from __future__ import annotations

import concurrent.futures as cf
import io
import itertools
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout's trunk/ (SPAGHETTY_REFERENCE_DIR names the checkout)
REF_TRUNK = os.path.join(os.environ.get("SPAGHETTY_REFERENCE_DIR", "/root/reference"), "trunk")
LIB = os.path.join(OUT, "libref_nests.so")

TRIPLES = None  # filled from the reference's nwchem_triples_usage()


def _load_emitter(path: str) -> dict:
    """Exec the generator module text up to its command-line driver (the
    ``compilers = [...]`` line), which only defines functions."""
    with open(path) as fh:
        text = fh.read()
    cut = text.index("\ncompilers = [")
    ns: dict = {"__name__": "spaghetty_ref_emitter"}
    exec(compile(text[:cut], path, "exec"), ns)
    return ns


def _patch(c_text: str) -> str:
    c_text = c_text.replace("const int f  = *factor;", "const double f  = *factor;")
    c_text = c_text.replace("const int g  = *acc_factor;", "const double g  = *acc_factor;")
    return c_text


def perm_str(p) -> str:
    return "".join(str(x) for x in p)


def generate() -> None:
    os.makedirs(OUT, exist_ok=True)
    g2 = _load_emitter(os.path.join(REF_TRUNK, "generator2.py"))
    g6 = _load_emitter(os.path.join(REF_TRUNK, "generator6.py"))
    triples = [list(p) for p in g6["nwchem_triples_usage"]()]

    perms4 = [list(p) for p in itertools.permutations("1234")]
    names4 = []
    for pi, p in enumerate(perms4):
        buf = io.StringIO()
        buf.write("#include <stddef.h>\n")
        for lo in perms4:
            name = "ref4_%s_loop_%s" % (perm_str(p), perm_str(lo))
            g2["generate_cfunction"](buf, name, "", True, p, lo)
            names4.append((perm_str(p), perm_str(lo), name))
        with open(os.path.join(OUT, "ref4_%s.c" % perm_str(p)), "w") as fh:
            fh.write(_patch(buf.getvalue()))

    perms6 = [list(p) for p in itertools.permutations([1, 2, 3, 4, 5, 6])]
    names6 = []
    chunk = 60
    for ci in range(0, len(perms6), chunk):
        buf = io.StringIO()
        buf.write("#include <stddef.h>\n")
        for p in perms6[ci:ci + chunk]:
            loops = [[1, 2, 3, 4, 5, 6]]
            if p in triples and p != [1, 2, 3, 4, 5, 6]:
                q = p[5]
                outer = [t for t in (1, 2, 3, 4, 5) if t != q]
                outer_out = [t for t in p if t not in (q, 6)]
                loops = [outer + [q, 6], outer + [6, q],
                         outer_out + [q, 6], outer_out + [6, q]]
                if loops[0] != [1, 2, 3, 4, 5, 6]:
                    loops.append([1, 2, 3, 4, 5, 6])
            seen = set()
            for lo in loops:
                key = perm_str(lo)
                if key in seen:
                    continue
                seen.add(key)
                name = "ref6_%s_loop_%s" % (perm_str(p), key)
                g6["generate_cfunction"](buf, name, "", True, p, lo)
                names6.append((perm_str(p), key, name))
        with open(os.path.join(OUT, "ref6_chunk%03d.c" % (ci // chunk)), "w") as fh:
            fh.write(_patch(buf.getvalue()))

    # dispatch table (our own code): name lookup by perm and loop order
    with open(os.path.join(OUT, "ref_table.c"), "w") as fh:
        fh.write("#include <string.h>\n#include <stddef.h>\n#include <omp.h>\n")
        fh.write("typedef void (*ref4_fn)(const double*, double*, const int*, const int*, "
                 "const int*, const int*, const double*, const double*);\n")
        fh.write("typedef void (*ref6_fn)(const double*, double*, const int*, const int*, "
                 "const int*, const int*, const int*, const int*, const double*, const double*);\n")
        for _, _, n in names4:
            fh.write("void %s(const double*, double*, const int*, const int*, const int*, "
                     "const int*, const double*, const double*);\n" % n)
        for _, _, n in names6:
            fh.write("void %s(const double*, double*, const int*, const int*, const int*, "
                     "const int*, const int*, const int*, const double*, const double*);\n" % n)
        fh.write("static const struct { const char *perm, *loop; ref4_fn fn; } T4[] = {\n")
        for p, lo, n in names4:
            fh.write('  {"%s", "%s", %s},\n' % (p, lo, n))
        fh.write("};\n")
        fh.write("static const struct { const char *perm, *loop; ref6_fn fn; } T6[] = {\n")
        for p, lo, n in names6:
            fh.write('  {"%s", "%s", %s},\n' % (p, lo, n))
        fh.write("};\n")
        fh.write("int ref_count(int rank) { return rank == 4 ? (int)(sizeof T4 / sizeof T4[0])"
                 " : (int)(sizeof T6 / sizeof T6[0]); }\n")
        fh.write("const char *ref_perm(int rank, int i) { return rank == 4 ? T4[i].perm : T6[i].perm; }\n")
        fh.write("const char *ref_loop(int rank, int i) { return rank == 4 ? T4[i].loop : T6[i].loop; }\n")
        # the OpenMP thread count of the nests, whatever OMP_NUM_THREADS the
        # process started with (a launcher may have set it to 1)
        fh.write("void ref_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }\n")
        fh.write("int ref_threads(void) { return omp_get_max_threads(); }\n")
        fh.write("int ref_call(int rank, int i, const double *u, double *s, const int *d,"
                 " double f, double g) {\n"
                 "  if (rank == 4) { T4[i].fn(u, s, d, d+1, d+2, d+3, &f, &g); return 0; }\n"
                 "  if (rank == 6) { T6[i].fn(u, s, d, d+1, d+2, d+3, d+4, d+5, &f, &g); return 0; }\n"
                 "  return -1;\n}\n")


def compile_lib(jobs: int | None = None) -> str | None:
    """Compile the generated C present in oracle/_ref into libref_nests.so."""
    if not os.path.isdir(OUT):
        return None
    srcs = sorted(f for f in os.listdir(OUT) if f.endswith(".c"))
    if "ref_table.c" not in srcs:
        return None
    newest = max(os.path.getmtime(os.path.join(OUT, s)) for s in srcs)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        try:
            subprocess.check_call(["true"])
            return LIB
        except Exception:
            pass
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = ["gcc", "-O3", "-std=gnu99", "-fopenmp", "-ffp-contract=off", "-fPIC", "-w"]

    def cc(s):
        obj = os.path.join(objdir, s[:-2] + ".o")
        subprocess.check_call(flags + ["-c", os.path.join(OUT, s), "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


def build() -> str | None:
    if os.path.isdir(REF_TRUNK):
        stamp = os.path.join(OUT, "ref_table.c")
        if not os.path.exists(stamp):
            generate()
    return compile_lib()


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--regenerate":
        generate()
    print(build())
