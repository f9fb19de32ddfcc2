"""Build recipe for the reference oracle (TEST INFRASTRUCTURE ONLY).

Compiles the reference's own main.cu as host C++ so that its per-chain code
(MH_simple_kernel, main.cu:679-813, and everything it calls) and its host
driver (main(), main.cu:1011-1257) can run on CPU cores:

  1. read main.cu from the reference checkout (default /root/reference; the
     GPU machine has no checkout and rebuilds from the copy made in step 2);
  2. write a substituted copy to oracle/_ref/src/gpr_ref_main.inc.  Every
     substitution is listed in SUBSTITUTIONS with the exact original line it
     replaces; the build refuses to run if a line does not match;
  3. compile oracle/ref_entry.cpp (which #includes that copy) with g++ into
     oracle/_ref/<variant>.so and an executable oracle/_ref/<variant>.cli.

The copy and all outputs live under oracle/_ref/, which git ignores: no
reference source is ever committed.  Variants are selected with -D knobs
documented in oracle/ref_shim.h.

Usage:  python oracle/build_ref.py [--pl 31] [--opset 0] [--philox 0]
                                   [--project-math 0] [--rw-sd 0] [--map-delta 0]
"""
import argparse
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("GPR_REFERENCE_DIR", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(OUT_DIR, "src")
GEN = os.path.join(SRC_DIR, "gpr_ref_main.inc")
KNOWN_MD5 = "d1100ae79713ae242a48571eace8fcc7"

# (1-based line in main.cu, exact original text (rstripped), replacement lines)
SUBSTITUTIONS = [
    (12, "#include <cuda_runtime.h>",
     ['#include "ref_shim.h"']),
    (17, '#include "math_constants.h" // Needed to define CUDART_NAN_F, CUDART_INF_F',
     ["/* math_constants.h: CUDART_NAN_F / CUDART_INF_F come from ref_shim.h */"]),
    (26, "const int PROGRAM_LENGTH = 31; // how many operations do we allow? This is the max index of the program array.",
     ["const int PROGRAM_LENGTH = GPR_REF_PL;"]),
    (27, "const int NCONSTANTS     = 31; // each op may use a constant if it wants (but most do not)",
     ["const int NCONSTANTS     = GPR_REF_PL;"]),
    (33, "const float P_PROPOSE_C_GEOMETRIC = 1.0; // how often do we propose setting a constant to an integer?",
     ["const float P_PROPOSE_C_GEOMETRIC = GPR_REF_P_GEOM;"]),
    (207, "#define RNG_DEF int& rx",
     ["#define RNG_DEF GPR_RNG_T& rx"]),
    (215, "   return rx = (rx * 1103515245 + 12345) & MY_RAND_MAX;",
     ["#if GPR_REF_PHILOX",
      "   return gpr_ref_philox_next(rx);",
      "#else",
      "   return rx = (rx * 1103515245 + 12345) & MY_RAND_MAX;",
      "#endif"]),
    (240, "    return sqrtf(-2.0*logf(u)) * sinf(2.0*PIf*v);",
     ["#if GPR_REF_PROJECT_MATH",
      "    return sqrtf(-2.0*gpr_rng_logf(u)) * gpr_rng_sinf(2.0*PIf*v);",
      "#else",
      "    return sqrtf(-2.0*logf(u)) * sinf(2.0*PIf*v);",
      "#endif"]),
    (253, "    return ceilf(logf(random_float(RNG_ARGS)) / log(r));",
     ["#if GPR_REF_PROJECT_MATH",
      "    return ceilf(gpr_rng_logf(random_float(RNG_ARGS)) / gpr_rng_logf(r));",
      "#else",
      "    return ceilf(logf(random_float(RNG_ARGS)) / log(r));",
      "#endif"]),
    (536, "    bayes_t prior = -PRIOR_MULTIPLIER * length * log((bayes_t)NOPS+1); // +1 for X (tree leaves, which count in the length)",
     ["    bayes_t prior = -PRIOR_MULTIPLIER * length * log((bayes_t)GPR_NOPS+1);"]),
    (691, "    int rx = random_seed + idx; // NOTE: We might want to call cuda_rand here once so that we don't have a bias from low seeds",
     ["    GPR_RNG_T rx; GPR_RNG_SEED(rx, random_seed, idx);"]),
    (718, "                        P[idx+i*N] = random_int(NOPS, RNG_ARGS);",
     ["                        P[idx+i*N] = GPR_OPMAP(random_int(GPR_NOPS, RNG_ARGS));"]),
    (781, "                        int order = random_int(C_MAX_ORDER-C_MIN_ORDER,RNG_ARGS)+C_MIN_ORDER; // what order of magnitude?",
     ["#if GPR_REF_RW",
      "                        C[i] = C[i] + (float)(GPR_REF_RW_SD) * random_normal(RNG_ARGS);",
      "#else",
      "                        int order = random_int(C_MAX_ORDER-C_MIN_ORDER,RNG_ARGS)+C_MIN_ORDER;"]),
    (782, "                        C[i] = C[i] + CONSTANT_SCALE * powf(10.0,order) * random_normal(RNG_ARGS);",
     ["                        C[i] = C[i] + CONSTANT_SCALE * powf(10.0,order) * random_normal(RNG_ARGS);",
      "#endif"]),
    (813, "}",
     ["}",
      "/* host launcher: one call of MH_simple_kernel per (block, thread), chains over OpenMP */",
      "static void gpr_ref_launch(int nb, int bs, int N, op* P, data_t* C, datum* D, int ndata,",
      "                           int steps, bayes_t* prior, bayes_t* likelihood, int random_seed) {",
      "    #pragma omp parallel for schedule(dynamic, 4)",
      "    for (long t = 0; t < (long)nb * bs; ++t) {",
      "        blockIdx.x = (unsigned)(t / bs); threadIdx.x = (unsigned)(t % bs); blockDim.x = (unsigned)bs;",
      "        MH_simple_kernel(N, P, C, D, ndata, steps, prior, likelihood, random_seed);",
      "    }",
      "}"]),
    # The reference formats expressions through 100-byte globals; expressions
    # longer than 99 characters overflow them and corrupt memory (observed:
    # garbled output, double free, a hang).  The oracle gives them room.
    (875, "char buf[2*PROGRAM_LENGTH+2][1000];",
     ["char buf[2*PROGRAM_LENGTH+2][1 << 16];"]),
    (876, "char lbuf[100], rbuf[100];",
     ["char lbuf[1 << 16], rbuf[1 << 16];"]),
    (1011, "int main(int argc, char** argv)",
     ["int gpr_ref_main(int argc, char** argv)"]),
    (1133, "    for(int i=0;i<PROGRAM_LENGTH*N;i++) host_P[i] = random_int(NOPS-1);",
     ["    for(int i=0;i<PROGRAM_LENGTH*N;i++) host_P[i] = GPR_OPMAP(random_int(GPR_NOPS-1));"]),
    (1160, "        MH_simple_kernel<<<N_BLOCKS,BLOCK_SIZE>>>(N, device_P, device_C, device_D, ndata, steps, device_prior, device_likelihood, rand());",
     ["        gpr_ref_launch(N_BLOCKS, BLOCK_SIZE, N, device_P, device_C, device_D, ndata, steps, device_prior, device_likelihood, rand());"]),
    (1219, "  \tbayes_t cutoff = host_posterior[int(N*RESAMPLE_QUANTILE)];",
     ["#if GPR_REF_MAPD",
      "  \tbayes_t cutoff = host_posterior[N-1] - (GPR_REF_MAP_DELTA);",
      "#else",
      "  \tbayes_t cutoff = host_posterior[int(N*RESAMPLE_QUANTILE)];",
      "#endif"]),
    (1225, "                for(int i=0;i<PROGRAM_LENGTH;i++) host_P[h+i*N] = random_int(NOPS-1);",
     ["                for(int i=0;i<PROGRAM_LENGTH;i++) host_P[h+i*N] = GPR_OPMAP(random_int(GPR_NOPS-1));"]),
    # host_D points into a std::vector; delete[] on it is a double free at exit.
    (1255, "    delete[] host_D;",
     ["    /* delete[] host_D: the vector owns that memory */"]),
    # main() ends without a return statement: implicit 0 for main, undefined
    # behaviour once it is renamed, so the renamed function returns 0 explicitly.
    (1257, "}",
     ["    return 0;", "}"]),
]


def extract(ref_dir=REF_DIR):
    """Write the substituted copy of main.cu to oracle/_ref/src/.  Returns the
    path, or None when there is neither a checkout nor an earlier copy."""
    src = os.path.join(ref_dir, "main.cu")
    if not os.path.exists(src):
        return GEN if os.path.exists(GEN) else None
    raw = open(src, "rb").read()
    md5 = hashlib.md5(raw).hexdigest()
    lines = raw.decode("latin-1").split("\n")
    subs = {ln: (orig, rep) for ln, orig, rep in SUBSTITUTIONS}
    out = []
    for i, line in enumerate(lines, start=1):
        if i in subs:
            orig, rep = subs[i]
            if line.rstrip() != orig.rstrip():
                raise RuntimeError(
                    "main.cu:%d does not match the expected text (md5 %s, expected %s):\n  got: %r\n  want: %r"
                    % (i, md5, KNOWN_MD5, line.rstrip(), orig))
            out.extend(rep)
        else:
            out.append(line)
    os.makedirs(SRC_DIR, exist_ok=True)
    body = "\n".join(out)
    header = "/* generated by oracle/build_ref.py from main.cu (md5 %s); not committed */\n" % md5
    if not os.path.exists(GEN) or open(GEN, encoding="latin-1").read() != header + body:
        with open(GEN, "w", encoding="latin-1") as f:
            f.write(header + body)
    return GEN


def variant_name(pl=31, opset=0, philox=0, project_math=0, rw_sd=0.0, map_delta=0.0):
    return "ref_pl%d_o%d_r%d_m%d_c%s_d%s" % (pl, opset, philox, project_math,
                                             ("%g" % rw_sd).replace(".", "p"),
                                             ("%g" % map_delta).replace(".", "p"))


def build(pl=31, opset=0, philox=0, project_math=0, rw_sd=0.0, map_delta=0.0,
          ref_dir=REF_DIR, force=False, verbose=False):
    """Build one variant.  Returns (so_path, cli_path) or None if the reference
    source is unavailable."""
    gen = extract(ref_dir)
    if gen is None:
        return None
    name = variant_name(pl, opset, philox, project_math, rw_sd, map_delta)
    so = os.path.join(OUT_DIR, name + ".so")
    cli = os.path.join(OUT_DIR, name + ".cli")
    deps = [gen, os.path.join(HERE, "ref_entry.cpp"), os.path.join(HERE, "ref_shim.h"),
            os.path.join(HERE, "..", "gpuropolis_gb300", "csrc", "gpr_rngmath.h"),
            os.path.join(HERE, "..", "gpuropolis_gb300", "csrc", "gpr_philox.h")]
    newest = max(os.path.getmtime(d) for d in deps)
    if (not force and os.path.exists(so) and os.path.exists(cli)
            and os.path.getmtime(so) >= newest and os.path.getmtime(cli) >= newest):
        return so, cli
    defs = ["-DGPR_REF_PL=%d" % pl, "-DGPR_REF_OPSET=%d" % opset,
            "-DGPR_REF_PHILOX=%d" % philox, "-DGPR_REF_PROJECT_MATH=%d" % project_math,
            "-DGPR_REF_RW=%d" % (rw_sd > 0), "-DGPR_REF_RW_SD=%r" % float(rw_sd),
            "-DGPR_REF_MAPD=%d" % (map_delta > 0), "-DGPR_REF_MAP_DELTA=%r" % float(map_delta)]
    # -fwrapv: the LCG (main.cu:215) relies on signed wrap-around.
    # -ffp-contract=off: same float results on x86 and Arm hosts.
    flags = ["g++", "-O3", "-std=gnu++17", "-fwrapv", "-ffp-contract=off", "-fopenmp", "-w",
             "-I", HERE, "-I", SRC_DIR] + defs
    entry = os.path.join(HERE, "ref_entry.cpp")
    cmds = [flags + ["-fPIC", "-shared", "-o", so + ".tmp", entry, "-lm"],
            flags + ["-DGPR_REF_WITH_MAIN=1", "-o", cli + ".tmp", entry, "-lm"]]
    for cmd in cmds:
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    os.replace(so + ".tmp", so)
    os.replace(cli + ".tmp", cli)
    return so, cli


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--pl", type=int, default=31)
    ap.add_argument("--opset", type=int, default=0)
    ap.add_argument("--philox", type=int, default=0)
    ap.add_argument("--project-math", type=int, default=0)
    ap.add_argument("--rw-sd", type=float, default=0.0)
    ap.add_argument("--map-delta", type=float, default=0.0)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    r = build(a.pl, a.opset, a.philox, a.project_math, a.rw_sd, a.map_delta, force=a.force, verbose=True)
    if r is None:
        print("reference source unavailable", file=sys.stderr)
        return 1
    print(r[0]); print(r[1])
    return 0


if __name__ == "__main__":
    sys.exit(main())
