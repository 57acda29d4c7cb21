/* ttsh.h — C ABI of libttsh, the GB300 (sm_103a) implementation of the TTSH3D timestep.
 *
 * The reference program (Sherlocked-L/Bacterial-Droplet, bacterial_droplet_12-16/TTSH3D.cu)
 * has no library interface: its path is the executable TTSH3D.out driven by run_cuda.pl,
 * reading data_<gpu_node>/input.dat and writing data_<gpu_node>/conf_<te>.dat. Each entry
 * point below replaces one host routine of that program (cited as file:line) so that a
 * thin main() — bacterial-droplet_gb300/shim/TTSH3D.cu — reproduces the program's
 * behaviour, and other callers (ctypes, cgo, JNI) can drive many droplets per launch.
 *
 * Conventions
 *   - Every call returns an int status: TTSH_OK (0) or a TTSH_E_* code; no exceptions cross
 *     the ABI. ttsh_strerror() maps a code to text; ttsh_last_error() gives the last message.
 *   - Host arrays are unpadded N^3 float64, x fastest: index (z*N + y)*N + x. The reference's
 *     device arrays carry an Nb-wide periodic halo (TTSH3D.cu:1127-1272); here the halo is
 *     implicit (periodic index wrap inside the kernels).
 *   - The library owns all device memory. A handle is used by one host thread at a time.
 *   - ttsh_step() is asynchronous on the handle's stream; get/reduce/write calls synchronise.
 */
#ifndef TTSH_H
#define TTSH_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TTSH_OK 0
#define TTSH_E_INVALID 1      /* bad argument or parameter value */
#define TTSH_E_IO 2           /* file could not be opened / written */
#define TTSH_E_PARSE 3        /* input.dat malformed or sentinel != -8848 */
#define TTSH_E_CUDA 4         /* a CUDA runtime call failed */
#define TTSH_E_NODEVICE 5     /* no CUDA device visible */
#define TTSH_E_NOMEM 6        /* device or host allocation failed */
#define TTSH_E_UNSTABLE 7     /* non-finite value detected by the watchdog */
#define TTSH_E_UNSUPPORTED 8  /* size or option not supported by this build */

#define TTSH_READ_SUCCESS (-8848) /* the reference's sentinel, TTSH3D.cu:748 */

/* The 33 tokens of input.dat, in file order (written by run_cuda.pl:53-86, read by
 * GetInput, TTSH3D.cu:696-752). Names and order are the reference's. */
typedef struct ttsh_input {
  int TimeScheme, RKStage, ExplImpi, AdapTime, ExpoData, InitCond, isSimplified, checkUnStable;
  int Nx, Ny, Nz, Nb;
  double h, dt0, T0, Ts, dte, dtVarC, dtMax;
  double mu, cA, alpha, beta, eta, La, kappa, lambda0, aPhi, kPhi, gamma, A, init0;
  int ReadSuccess;
} ttsh_input;

/* Build-defined options that input.dat does not carry (kept in a separate struct so that
 * input.dat stays byte-compatible with run_cuda.pl and readDraw.py). */
#define TTSH_K2_REFERENCE 0   /* continuous k^2, k2[0] = 1 (initPoissonSolver, TTSH3D.cu:1088-1124) */
#define TTSH_K2_DISCRETE 1    /* modified wavenumber of the 27-point gradient: exactly solenoidal */
#define TTSH_QUIRK_STALE_HALO 1 /* divergence of u*, P* sees last step's halo (getRHS :369-371) */
typedef struct ttsh_ext {
  double zeta;     /* active stress -zeta * div(phi P P); 0 = the reference's physics */
  double R, xi;    /* droplet radius and interface width of ttsh_init_droplet */
  uint64_t seed;   /* polarisation seed of ttsh_init_droplet */
  int precision;   /* 64 = FP64 fields and FFT, 32 = FP32 fields and FFT */
  int k2_mode;     /* TTSH_K2_REFERENCE or TTSH_K2_DISCRETE */
  int quirks;      /* bitmask of TTSH_QUIRK_* (default TTSH_QUIRK_STALE_HALO) */
  int form;        /* TTSH_FORM_AUTO, TTSH_FORM_PLAIN or TTSH_FORM_FUSED (same for all droplets) */
} ttsh_ext;
#define TTSH_FORM_AUTO 0   /* fused kernels where supported (FP32, N a multiple of 32), else plain */
#define TTSH_FORM_PLAIN 1  /* one thread per site, the reference's arithmetic order (FP64 or FP32) */
#define TTSH_FORM_FUSED 2  /* fused FP32 kernels; TTSH_E_UNSUPPORTED where they do not apply */

typedef struct ttsh_stats {
  double mass;       /* sum(phi) h^3, FP64 reduction */
  double max_div_u;  /* max |sum_a D_a u_a| after the last projection, FP64 */
  double max_abs_u;  /* max |u_a| */
  double T;          /* simulated time */
  int64_t steps;     /* steps taken since creation */
  int nonfinite;     /* 1 if any NaN/Inf was seen in phi, P or u */
  int reserved;
} ttsh_stats;

typedef struct ttsh_sim ttsh_sim;

/* GetInput (TTSH3D.cu:696-752): parse the 33 whitespace-separated tokens of input.dat.
 * Returns TTSH_E_PARSE when a token is missing or the sentinel is not -8848 (the reference
 * prints "Error while reading the input file!" and skips the run, :748-751, :270). */
int ttsh_read_input(const char* path, ttsh_input* out);

/* Fill `out` with the reference defaults of run_cuda.pl:7-44 (N = 64). */
void ttsh_default_input(ttsh_input* out);
void ttsh_default_ext(ttsh_ext* out);

/* MemAlloc + initPoissonSolver + cudaMemcpyToSymbol(p) (TTSH3D.cu:1127-1272, :1088-1124,
 * :761): one droplet. Requires Nx == Ny == Nz (the reference's FFT plan is valid for cubes
 * only, :1123). `device` < 0 selects the current device. */
int ttsh_create(const ttsh_input* in, const ttsh_ext* ext, int device, ttsh_sim** out);

/* Many independent droplets advanced together (one launch per kernel per size group).
 * `in` and `ext` are arrays of n entries; sizes may differ between instances. */
int ttsh_batch_create(const ttsh_input* in, const ttsh_ext* ext, int n, int device, ttsh_sim** out);

/* Use a caller stream (cudaStream_t passed as void*); NULL = the library's own stream. */
int ttsh_set_stream(ttsh_sim* s, void* stream);

/* InitConf (TTSH3D.cu:755-896), host -> device: set instance `inst`'s state from host
 * arrays. P and u are 3*N^3 (component-major: x, y, z). ustar/Pstar may be NULL (zeros);
 * they seed the previous-step halo of quirk Q2. */
int ttsh_set_state(ttsh_sim* s, int inst, const double* phi, const double* P, const double* u,
                   const double* ustar, const double* Pstar);

/* The build-defined initial condition (host only, no GPU needed): phi = (1 - tanh((r-R)/xi))/2
 * centred at (N/2,N/2,N/2); P = unit vectors where phi > 0.5 with directions uniform on the
 * sphere from `seed` (counter-based), 3 Jacobi passes (self + 6 face neighbours, periodic),
 * then zero where phi <= 0.5; `angular_noise` > 0 adds Gaussian angular noise (radians) to
 * the initial directions. Replaces InitConf's time(0)-seeded noise (TTSH3D.cu:801-824). */
int ttsh_init_droplet(int N, double h, double R, double xi, uint64_t seed, double angular_noise,
                      double* phi, double* P);

/* InitConf's own initial state (TTSH3D.cu:755-896), host only: InitCond == 1 draws uniform noise
 * init0*(U-1/2) for u, u*, P, P* (and two discarded draws for p_v, p_p) from
 * std::default_random_engine(seed), 14 draws per site, x outer / y / z inner as the reference
 * does, and phi = (1 - tanh((r - Nx/4)*2))/2; InitCond == 0 reads vx, vy (2 columns per site, the
 * same loop order) from `conf0_path` (the reference's data/conf_<t0>.dat). Arrays as
 * ttsh_set_state's; P, u, ustar, Pstar are 3*N^3. */
int ttsh_init_reference(const ttsh_input* in, unsigned seed, const char* conf0_path, double* phi, double* P,
                        double* u, double* ustar, double* Pstar);

/* forEach.pl's sweep as one batched run: the reference runs one TTSH3D.out per parameter set
 * (forEach.pl:33-131, run_cuda.pl:136). Each of the n directories holds an input.dat; all droplets
 * advance together (one launch per kernel per size group), each with its own constants, dt, dte
 * and Ts, starting from ttsh_init_reference(seed + i), and each writes its conf_<te>.dat files
 * into its own directory at the times TTSH3D.out would (conf_0.dat first when T0 == 0). A droplet
 * whose T has passed its Ts stops writing; the batch ends when all have. `ext` may be NULL
 * (defaults) and applies to every droplet. */
int ttsh_run_dirs(const char* const* dirs, int n, const ttsh_ext* ext, uint64_t seed, int device);

/* EEuler x nsteps (TTSH3D.cu:347-359, run/evolve :336-343, :311-331): asynchronous. */
int ttsh_step(ttsh_sim* s, int nsteps);

/* Block until all queued work on the handle's stream is done; returns a CUDA error if any. */
int ttsh_sync(ttsh_sim* s);

/* Device -> host copies of ExpoConf (TTSH3D.cu:904-963): any pointer may be NULL.
 * P, u, ustar, Pstar are 3*N^3; p_v and p_p are the last projection's pressures.
 * Host arrays of ttsh_set_state / ttsh_get_state / ttsh_get_provisional in page-locked memory
 * (cudaHostAlloc, cudaHostRegister, torch's pin_memory) are read and written in place by the
 * device's conversion kernels; pageable arrays are staged through device memory by the copy
 * engines. Both give the same values. */
int ttsh_get_state(ttsh_sim* s, int inst, double* phi, double* P, double* u, double* p_v, double* p_p);
int ttsh_get_provisional(ttsh_sim* s, int inst, double* ustar, double* Pstar);

/* FP64 diagnostics (new; the reference has none): mass, divergence, non-finite watchdog. */
int ttsh_reduce(ttsh_sim* s, int inst, ttsh_stats* out);

/* The same diagnostics for every droplet of the handle in one pass per size group and one
 * device-to-host copy: out[i] for each instance i. TTSH_STATS_MASS computes only the FP64 mass
 * and the non-finite flag of phi (max_div_u and max_abs_u are set to -1): the per-step monitor of
 * a batch. TTSH_STATS_ALL is ttsh_reduce for every droplet. */
#define TTSH_STATS_ALL 0
#define TTSH_STATS_MASS 1
int ttsh_reduce_all(ttsh_sim* s, int what, ttsh_stats* out);

/* Asynchronous form of ttsh_reduce_all for diagnostics recorded every step without stalling
 * the GPU (the reference prints nothing per step; its ExpoConf, TTSH3D.cu:899-1014, is the only
 * read-back): enqueues the diagnostics of every droplet on the handle's stream and their copy
 * into `partials` (caller-owned host memory of ttsh_partials_size(s) doubles; page-locked memory
 * makes the copy asynchronous), and returns without waiting. After ttsh_sync (or any call that
 * waits for the stream), ttsh_stats_from_partials turns a filled buffer into per-droplet
 * ttsh_stats, whose steps and T are the values at the call. A buffer must not be reused before its
 * copy has completed. */
size_t ttsh_partials_size(const ttsh_sim* s);
int ttsh_reduce_all_async(ttsh_sim* s, int what, double* partials);
int ttsh_stats_from_partials(const ttsh_sim* s, const double* partials, ttsh_stats* out);

/* ExpoConf (TTSH3D.cu:899-1014): write the snapshot text file of instance `inst` at `path`:
 * one line per site, y outer, x, z inner; columns "vx vy vz px py pz phi" printed as
 * fixed with 15 decimals (ExpoData == 1) or "vx vy " (ExpoData == -1). */
int ttsh_write_conf(ttsh_sim* s, int inst, const char* path);
/* ttsh_write_conf_async — ExpoConf (TTSH3D.cu:899-1014) without stopping the steps: enqueues the
 * snapshot of droplet `inst` on the handle's stream and returns. The fields are converted to FP64
 * straight into a page-locked host buffer of the handle, in stream order, and a host thread
 * formats and writes the file (the same bytes as ttsh_write_conf) while later steps run. One
 * snapshot is in flight at a time: a second call first waits for the previous one. */
int ttsh_write_conf_async(ttsh_sim* s, int inst, const char* path);
/* Waits for the snapshot in flight, if any, and returns its status. ttsh_destroy waits too. */
int ttsh_conf_wait(ttsh_sim* s);

/* Same formatter on host arrays (no GPU): for writing conf files from any source. */
int ttsh_format_conf(int N, int expo_data, const double* phi, const double* P, const double* u,
                     const char* path);

/* readDraw.py's reductions of one snapshot, on the device (so no 3D text file is needed):
 * centroid[3] = the phi-weighted mean (y, x, z) in FP64 (calculate_centroid, readDraw.py:30-52,
 * which returns the int() of these), index[3] = those int() values, and slices = 9*N*N doubles,
 * each a [y][x] plane at z = index[2]: vx, vy, vz, px, py, pz, phi, then the vorticities
 * d1xO4(vy) - d1yO4(vx) and d1xO4(py) - d1yO4(px) (readDraw.py:222-237, op.py:3-13).
 * The centroid sums are FP64 in a fixed (parallel) order; readDraw sums sequentially, so index
 * can differ from readDraw's only when a mean lies within ~1e-12 of an integer. */
int ttsh_snapshot_slice(ttsh_sim* s, int inst, double* centroid, int* index, double* slices);

/* Checkpoint / resume (replaces the reference's T0 > 0 restart, TTSH3D.cu:769-797, which reads
 * only vx, vy of InitCond == 0 from data/conf_<t0>.dat). The file holds T and phi, P, u, u*, P*
 * (u*, P* feed the next step's stale halo) as the device stores them (FP32 or FP64), so a run
 * resumed from it continues bit for bit. Layout: "TTSHCKP1", int32 version 1, int32 N, int32
 * precision, int32 extra, double T, int64 steps, then 13 + extra arrays of N^3 (phi, P x3, u x3,
 * u* x3, P* x3; the fused FP32 form adds its phi-update compensation, extra = 1).
 * The pressures are not stored: they are recomputed by the next step. */
int ttsh_save_checkpoint(ttsh_sim* s, int inst, const char* path);
int ttsh_load_checkpoint(ttsh_sim* s, int inst, const char* path);

/* MemFree + cufftDestroy (TTSH3D.cu:280-281, :1275-1419). */
void ttsh_destroy(ttsh_sim* s);

const char* ttsh_strerror(int code);
const char* ttsh_last_error(void);

/* Instances, their sizes, the simulated time. */
int ttsh_num_instances(const ttsh_sim* s);
int ttsh_instance_n(const ttsh_sim* s, int inst);
double ttsh_time(const ttsh_sim* s);

/* Timing helper for benchmarks: runs nsteps steps with a CUDA event pair around every kernel
 * of the step and returns, per kernel class, the mean device time per step in ms.
 * names[i] point to static strings. Returns the number of classes written (<= cap). */
int ttsh_profile_kernels(ttsh_sim* s, int nsteps, int cap, const char** names, double* ms_per_step,
                         int64_t* launches_per_step);

/* sizeof(ttsh_input) for which == 0, sizeof(ttsh_ext) for 1, sizeof(ttsh_stats) for 2,
 * sizeof(ttsh_tuning) for 3, else -1: lets a caller that re-declares the structures (the
 * TTSH3D.cu shim) check the layout. */
int ttsh_struct_size(int which);

/* Autotuner — no counterpart in the reference (whose tile shapes are fixed by its launch
 * configuration, TTSH3D.cu:224-235, and whose FFT plan is cuFFT's, :1123). The choices are made
 * per group of droplets of equal N (one launch per kernel per group):
 *   the FFT: register-resident kernels (where the size has them; per axis, or x and y of a plane
 *   in one launch) or the shared-memory Stockham passes, with their lines per CTA and the order
 *   of the radix plan;
 *   the fused FP32 kernels: the z-extent of a CTA's tile (z-planes per CTA) of each of the three.
 * None of them changes results except the FFT choice (rounding order only). */
typedef struct {
  int N;           /* droplet size of the group */
  int n;           /* droplets in the group */
  int fft_kind;    /* register-resident kernels where the size has them: 0 one launch per axis
                      pass, 2 x and y of each plane in one launch; 1 Stockham */
  int fft_lb;      /* Stockham lines per CTA; 0 = the largest that fits */
  int nstages;     /* Stockham radix plan: radix[0..nstages-1], each 2, 3, 4 or 5, product N */
  int radix[16];
  int zc[3];       /* z-planes per CTA of fused_rhs, fused_div, fused_correct (fused form);
                      0: a persistent grid (the CTAs that fit on the device at once), each CTA
                      sweeping an equal contiguous share of the group's (droplet, tile, plane) sites */
  double ms[4];    /* measured per launch: FFT (5 passes), fused_rhs, fused_div, fused_correct;
                      0 where not measured (taken from a cache, or set by the caller) */
} ttsh_tuning;

/* Number of groups (distinct N) of the instance. */
int ttsh_num_groups(const ttsh_sim* s);
/* The configuration group `group` runs with. */
int ttsh_get_tuning(const ttsh_sim* s, int group, ttsh_tuning* out);
/* Applies a configuration to group `group` (N and n must match the group); TTSH_E_INVALID for
 * a configuration the kernels do not support. Takes effect from the next step. */
int ttsh_set_tuning(ttsh_sim* s, int group, const ttsh_tuning* in);
/* Times the candidates of every group on the instance's own fields and keeps the fastest. The
 * state (phi, P, u, u*, P*, the pressures and T) is left as it was. With cache_path non-NULL,
 * groups with an entry for this GPU, precision, form, N and group size in that text file take
 * it without timing, and the choices of the others are appended to it. */
int ttsh_autotune(ttsh_sim* s, const char* cache_path);

/* Launch count of one step (kernels of this library). */
int ttsh_launches_per_step(const ttsh_sim* s);

/* Largest grid ttsh_step_noalloc accepts (its fixed working memory is sized for it). */
#define TTSH_NOALLOC_MAX_N 32

/* ttsh_step_noalloc — no counterpart in the reference (which allocates all its arrays in
 * MemAlloc). For callers that cannot allocate device memory: their device memory belongs to
 * another allocator or is capped per process, or they cannot afford cudaFree's device-wide
 * wait. Advances one droplet `nsteps` explicit steps in FP64 (the plain form, the same kernels
 * and results as ttsh_step) and allocates nothing: the caller passes DEVICE pointers to its
 * own FP64 arrays, and the step's working memory is one fixed array inside libttsh
 * (about 5.8 MB, present on every GPU that loads the library until the process exits).
 *   phi (N^3), P, u (3*N^3): state, updated in place.
 *   ustar, Pstar (3*N^3): on entry the previous step's u*, P* (zeros at the start; they feed the
 *     stale-halo divergence), on return this call's last u*, P*.
 *   p_v, p_p (N^3): outputs, the last projection's pressures (untouched when nsteps == 0).
 *   stream: cudaStream_t as void* (NULL = legacy default stream). The call enqueues its work on
 *     that stream and returns without waiting for it or for earlier work (the tables and the
 *     droplet descriptor travel as a kernel parameter, not through a host-to-device copy).
 * Rejects N > TTSH_NOALLOC_MAX_N, non-cubic grids and precision != 64 with TTSH_E_UNSUPPORTED.
 * All calls share the working array and leave its contents behind (nothing in it must start
 * at zero); calls whose GPU work overlaps race on it and must be serialised by the caller.
 * The first call on a device looks up the array's device address; the first call for a size on
 * a device also sets kernel attributes, fills a constant table and waits for the device to
 * finish. Make those first calls before starting any stream capture on the calling thread. */
int ttsh_step_noalloc(const ttsh_input* in, const ttsh_ext* ext, int nsteps, double* phi, double* P, double* u,
                      double* ustar, double* Pstar, double* p_v, double* p_p, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TTSH_H */
