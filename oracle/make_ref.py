"""Recipe: build the reference's own TTSH3D program, patched only at its edges, into oracle/_ref/.

TEST INFRASTRUCTURE ONLY. The generated source and binary are the checker's
second oracle (the reference's own CUDA step, run on the GPU) and the timed
reference arm of bench.py. Nothing here is part of the product.

Where the reference sources exist (the development container), the script reads
bacterial_droplet_12-16/TTSH3D.cu, applies the patches below and writes
oracle/_ref/TTSH3D_ref.cu. The generated file is git-ignored and travels with
the working tree, so a machine without the reference sources compiles the
previously generated file. The step itself (getRHS, getVStar, getP, getStream,
getVNew, the stencils, BounPeriU, initPoissonSolver) is left byte-identical.

Patches (each anchor must occur exactly once):
  0. the RNG seed (TTSH3D.cu:40) is $TTSH_SEED when set, else time(0) as in the reference.
  1. InitConf (TTSH3D.cu:755-896): after the reference's own random init, the
     fields are overwritten from data_<gpu_node>/init.bin when that file exists
     (int32 N, int32 nfields, then nfields unpadded N^3 float64 arrays in the
     order phi px py pz vx vy vz vxs vys vzs pxs pys pzs pv pp; absent fields = 0).
  2. evolve (TTSH3D.cu:290-332): the step loop is timed with cudaDeviceSynchronize
     + steady_clock after TTSH_REF_WARMUP steps (environment, default 0), and
     one line "TTSH_REF_TIMING steps=<n> seconds=<s>" is printed.
  3. main (TTSH3D.cu:263-287): after evolve(), all 15 state fields are copied
     to the host and written to data_<gpu_node>/final.bin in the init.bin layout.
Build line: the reference's own (run_cuda.pl:4), nvcc -std=c++14 --cudart=shared
-lcufft, with no -arch (stock code path: compute_75 PTX, JIT-compiled on the GPU).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference checkout this recipe reads (development container only; never on the GPU machine).
REF_ROOT = os.environ.get("TTSH_REFERENCE_ROOT", "/root/reference")
REF_DIR = os.path.join(REF_ROOT, "bacterial_droplet_12-16")
REF_SRC = os.path.join(REF_DIR, "TTSH3D.cu")
GEN = os.path.join(OUT, "TTSH3D_ref.cu")
BIN = os.path.join(OUT, "ttsh_ref.out")

FIELDS = ["phi", "px", "py", "pz", "vx", "vy", "vz", "vx_star", "vy_star", "vz_star",
          "px_star", "py_star", "pz_star", "p_v", "p_p"]

HELPERS = r'''
// ---- added by oracle/make_ref.py: binary init / dump helpers (not part of the step) ----
#include <chrono>
#include <cstdlib>
static real* ttshref_host_field(int c) {
  real* tab[15] = {F.phi, F.px, F.py, F.pz, F.vx, F.vy, F.vz, F.vx_star, F.vy_star, F.vz_star,
                   F.px_star, F.py_star, F.pz_star, F.p_v, F.p_p};
  return tab[c];
}
static real* ttshref_dev_field(int c) {
  real* tab[15] = {f.phi, f.px, f.py, f.pz, f.vx, f.vy, f.vz, f.vx_star, f.vy_star, f.vz_star,
                   f.px_star, f.py_star, f.pz_star, f.p_v, f.p_p};
  return tab[c];
}
static size_t ttshref_pidx(int x, int y, int z) {
  return (size_t)(P.Nx + 2 * P.Nb) * (P.Ny + 2 * P.Nb) * (z + P.Nb) + (size_t)(P.Nx + 2 * P.Nb) * (y + P.Nb) + x + P.Nb;
}
static void ttshref_load_init() {
  std::string fn = "data_" + to_string(gpu_node) + "/init.bin";
  FILE* fp = fopen(fn.c_str(), "rb");
  if (!fp) return;
  int hdr[2] = {0, 0};
  if (fread(hdr, sizeof(int), 2, fp) != 2 || hdr[0] != P.Nx || hdr[0] != P.Ny || hdr[0] != P.Nz) {
    cout << "TTSH_REF_ERROR bad init.bin header" << endl;
    fclose(fp);
    exit(3);
  }
  size_t n = (size_t)P.Nx * P.Ny * P.Nz;
  std::vector<double> buf(n);
  for (int c = 0; c < 15; ++c) {
    bool have = c < hdr[1];
    if (have && fread(buf.data(), sizeof(double), n, fp) != n) {
      cout << "TTSH_REF_ERROR short init.bin" << endl;
      fclose(fp);
      exit(3);
    }
    real* dst = ttshref_host_field(c);
    for (int z = 0; z < P.Nz; ++z)
      for (int y = 0; y < P.Ny; ++y)
        for (int x = 0; x < P.Nx; ++x)
          dst[ttshref_pidx(x, y, z)] = have ? buf[((size_t)z * P.Ny + y) * P.Nx + x] : 0.0;
  }
  fclose(fp);
  cout << "TTSH_REF_INIT loaded " << hdr[1] << " fields" << endl;
}
static void ttshref_dump_final() {
  std::string fn = "data_" + to_string(gpu_node) + "/final.bin";
  FILE* fp = fopen(fn.c_str(), "wb");
  if (!fp) return;
  int hdr[2] = {P.Nx, 15};
  fwrite(hdr, sizeof(int), 2, fp);
  size_t n = (size_t)P.Nx * P.Ny * P.Nz;
  std::vector<double> buf(n);
  for (int c = 0; c < 15; ++c) {
    real* h = ttshref_host_field(c);
    cudaMemcpy(h, ttshref_dev_field(c), P.BSize, cudaMemcpyDeviceToHost);
    for (int z = 0; z < P.Nz; ++z)
      for (int y = 0; y < P.Ny; ++y)
        for (int x = 0; x < P.Nx; ++x) buf[((size_t)z * P.Ny + y) * P.Nx + x] = h[ttshref_pidx(x, y, z)];
    fwrite(buf.data(), sizeof(double), n, fp);
  }
  fclose(fp);
  cout << "TTSH_REF_DUMP " << fn << endl;
}
// ---- end of added helpers ----
'''

PATCHES = [
    # 0. seed: $TTSH_SEED when set, else the reference's time(0) (TTSH3D.cu:40)
    ("int seed = time(0);\n", "int seed = getenv(\"TTSH_SEED\") ? atoi(getenv(\"TTSH_SEED\")) : time(0);\n"),
    ('#include "cuda_runtime.h"\n', '#include <cstdlib>\n#include "cuda_runtime.h"\n'),
    # 1. helpers after the global declarations (before main)
    ("//=======================================================================\nint main()\n",
     HELPERS + "//=======================================================================\nint main()\n"),
    # 1b. load the binary init at the end of the host-side init loop in InitConf
    ("  // Still need to get vortex\n",
     "  ttshref_load_init();\n  // Still need to get vortex\n"),
    # 2. timing around the step loop in evolve
    ("  while (iStop == 0)\n  {\n\n    // Evolution\n    run();\n",
     "  int ttshref_warm = getenv(\"TTSH_REF_WARMUP\") ? atoi(getenv(\"TTSH_REF_WARMUP\")) : 0;\n"
     "  long ttshref_steps = 0;\n"
     "  cudaDeviceSynchronize();\n"
     "  auto ttshref_t0 = std::chrono::steady_clock::now();\n"
     "  while (iStop == 0)\n  {\n\n    // Evolution\n"
     "    if (ttshref_steps == ttshref_warm) { cudaDeviceSynchronize(); ttshref_t0 = std::chrono::steady_clock::now(); }\n"
     "    run();\n    ++ttshref_steps;\n"),
    ("    // Check.\n    if (T > P.Ts)\n    {\n      iStop = 1;\n    }\n  }\n}\n",
     "    // Check.\n    if (T > P.Ts)\n    {\n      iStop = 1;\n    }\n  }\n"
     "  cudaDeviceSynchronize();\n"
     "  double ttshref_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - ttshref_t0).count();\n"
     "  cout << endl << \"TTSH_REF_TIMING steps=\" << (ttshref_steps - (ttshref_steps > ttshref_warm ? ttshref_warm : 0))"
     " << \" seconds=\" << ttshref_s << endl;\n}\n"),
    # 3. dump after evolve
    ("    evolve();\n    cufftDestroy(plan);\n",
     "    evolve();\n    ttshref_dump_final();\n    cufftDestroy(plan);\n"),
]


def generate(src_path: str = REF_SRC, out_path: str = GEN) -> str:
    with open(src_path, "r", encoding="utf-8", errors="surrogateescape") as fh:
        src = fh.read()
    for anchor, repl in PATCHES:
        n = src.count(anchor)
        if n != 1:
            raise RuntimeError("patch anchor found %d times: %r" % (n, anchor[:60]))
        src = src.replace(anchor, repl)
    os.makedirs(os.path.dirname(out_path), exist_ok=True)
    with open(out_path, "w", encoding="utf-8", errors="surrogateescape") as fh:
        fh.write(src)
    return out_path


def compile_ref(gen: str = GEN, out: str = BIN) -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = out + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc, "-std=c++14", "--cudart=shared", gen, "-o", tmp, "-lcufft"],
                          stdout=subprocess.DEVNULL)
    os.replace(tmp, out)
    return out


def build(compile_binary: bool = True) -> str | None:
    """Generate (when the reference sources are present) and compile. Returns the binary path or None."""
    if os.path.exists(REF_SRC):
        generate()
    if not os.path.exists(GEN):
        return None
    if not compile_binary:
        return GEN
    if not os.path.exists(BIN) or os.path.getmtime(BIN) < os.path.getmtime(GEN):
        compile_ref()
    return BIN


if __name__ == "__main__":
    print(build(compile_binary="--no-compile" not in sys.argv))
