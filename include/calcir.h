/*
 * calcir.h -- C ABI of the GB300 (sm_103a) calcIR spectroscopy hot path.
 *
 * The reference (nicholashestand/calcIR) is one executable, `calcIR.exe input.inp`,
 * with no library API.  Each entry point below replaces one stage of its per-frame
 * loop; the file:line after each declaration names the reference code it stands in
 * for (paths are relative to the reference project root).
 *
 * Conventions
 *  - Every function returns an int status: CIR_OK (0) or a negative CIR_ERR_* code.
 *    cir_last_error() returns a message for the calling thread's last failure.
 *    (The reference prints and calls exit(EXIT_FAILURE), calcIR.h:44-46.)
 *  - Array arguments of the stage functions may be HOST or DEVICE pointers.  Device
 *    pointers are used in place and the call is asynchronous on the context's stream;
 *    host arrays are staged through the context and the call returns after the copy back.
 *  - N = nchrom = nmol * nchrom_mol chromophores.  Matrices are N x N float32.  A complex
 *    matrix is stored as interleaved (re, im) float32 pairs, row-major.
 *  - Units follow the reference: positions in nm, times in ps, energies in cm^-1.
 *  - Nothing here falls back to the CPU: without a usable CUDA device cir_create fails
 *    with CIR_ERR_NODEVICE.
 */
#ifndef CALCIR_H_
#define CALCIR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CIR_VERSION_STRING "0.1.0"

/* status codes */
#define CIR_OK              0
#define CIR_ERR_ARG        -1   /* null pointer, size or value out of range            */
#define CIR_ERR_CUDA       -2   /* CUDA runtime error                                   */
#define CIR_ERR_NOMEM      -3   /* host or device allocation failed                     */
#define CIR_ERR_NOCONVERGE -4   /* eigensolver reached its sweep cap                    */
#define CIR_ERR_IO         -5   /* file could not be opened, read or written            */
#define CIR_ERR_PARSE      -6   /* unknown model / species / map in the input           */
#define CIR_ERR_STATE      -7   /* call out of order                                    */
#define CIR_ERR_NONFINITE  -8   /* NaN or Inf in the positions, box or (host) matrices   */
#define CIR_ERR_NODEVICE   -9   /* no CUDA device could be used                          */

/* arithmetic of the propagation and correlation GEMMs */
#define CIR_PREC_FP32   0   /* plain drop-in form: FP32 everywhere                     */
#define CIR_PREC_TF32   1   /* tensor-core TF32 GEMMs, FP32 accumulation               */
#define CIR_PREC_BF16X3 2   /* tensor-core 3-pass split-BF16 GEMMs, FP32 accumulation  */

#define CIR_STRLEN 256

/* Run parameters.  The first block mirrors the 19 input.inp keys with the reference
 * defaults (calcIR.cu:36-59, parsed by ir_init calcIR.cu:1539-1643).  imodel/ispecies
 * are decoded from model/species by cir_params_finalize (calcIR.cu:324-339).  The
 * synth_* and engine keys are additions; the reference parser would warn and ignore them. */
typedef struct cir_params {
    char  xtcf[CIR_STRLEN];        /* trajectory: a .cirtrj file or "synthetic"        */
    char  outf[CIR_STRLEN];        /* output file prefix                               */
    char  cptf[CIR_STRLEN];        /* accepted and unused, as in the reference          */
    char  model[CIR_STRLEN];       /* tip4p | e3b2 (imodel 0), tip4p2005 | e3b3 (1)     */
    char  species[CIR_STRLEN];     /* H2O | HOD/D2O | HOD/H2O | D2O                      */
    int   ntcfpoints;
    int   nsamples;
    float sampleEvery;             /* ps between time origins                          */
    int   omegaStep;               /* cm^-1, integer as in the reference                */
    int   natom_mol;
    int   nchrom_mol;
    int   nzeros;                  /* zero padding of the TCF before the transform      */
    int   map;                     /* 0 Gruenbaum 2013, 1 Li-Skinner 2010              */
    float dt;                      /* ps between TCF points                            */
    float t1;                      /* ps, vibrational relaxation time                  */
    float avef;                    /* cm^-1 subtracted from the diagonal               */
    float beginTime;               /* ps                                               */
    float omegaStart;
    float omegaStop;
    /* decoded */
    int   imodel;
    int   ispecies;
    /* synthetic frame source (used when xtcf == "synthetic") */
    int   synth_nmol;
    int   synth_seed;
    float synth_frame_dt;          /* ps between generated frames (default 0.010)      */
    float synth_sigma_trans;       /* nm per axis per frame (default 0.003)            */
    float synth_sigma_rot;         /* degrees per frame (default 3)                    */
    /* engine options */
    int   precision;               /* CIR_PREC_*                                       */
    int   batch_frames;            /* frame-steps per eigensolver batch, 0 = automatic */
    int   verbose;                 /* 0 silent, 1 reference-style progress on stdout   */
    int   cuda_graphs;             /* 1: replay the per-step launches from captured CUDA graphs */
    int   autotune;                /* 1: time the GEMM tile shapes once per problem shape      */
    /* options of the run that give the same results by less work; off by default, so that
       the default run does the reference's work (full F propagation, one eigensolve per
       origin and step) */
    int   propagate_vectors;       /* 1: propagate psi_a = F m_a(0) (9 complex vectors) instead of F */
    int   share_frames;            /* 1: one eigensolve per distinct frame when origins overlap      */
    /* precision option, off by default: steps of FP64 refinement of every eigendecomposition
       (Rayleigh quotients, first-order eigenvector correction and re-orthogonalisation;
       2 takes FP32 / split-BF16 eigenpairs to the accuracy of FP32 storage) */
    int   refine_eigen;
    /* fault drills for tests, 0 (off) by default: each makes a bounded wait or iteration
       cap of the GPU path run out on purpose, so that its error status can be checked
       without faulting or hanging the GPU */
    int   test_stall_gemm;         /* 1: the persistent split-BF16 GEMM withholds its first tile's
                                      completion; its bounded waits (shortened to 2^14 polls) run
                                      out and the call returns CIR_ERR_CUDA ("timed out") */
    int   test_sweep_cap;          /* > 0: QR sweeps allowed per divide-and-conquer leaf; a cap the
                                      leaves cannot meet makes cir_eigh return CIR_ERR_NOCONVERGE */
} cir_params;

/* Whole-job results, caller-owned host arrays sized by cir_result_sizes. */
typedef struct cir_result {
    double *tcf_ir, *tcf_vv, *tcf_vh;   /* [2*ntcfpoints] (re,im), damped and /nsamples,
                                           the values of the *_{ir,vv,vh}{r,i}tcf.dat files */
    float  *omega;                      /* [nomega] omegaStart + omegaStep*i             */
    float  *sw, *pw, *rw, *rmw;         /* [nomega] _spdn, _Pw, _Rw, _Rmw                 */
    float  *ls_omega, *ls_ir, *ls_vv, *ls_vh;   /* [nls] _irls, _vvls, _vhls rows, descending omega */
    int     nls;                        /* out: lineshape rows                            */
    long long bins_out_of_range;        /* out: eigenvalues outside [omegaStart,omegaStop];
                                           the reference writes those out of bounds
                                           (calcIR.cu:529-537), here they are counted     */
    double  frame_steps_per_s;          /* out: frame-steps / device seconds of the loop */
} cir_result;

typedef struct cir_stats {
    long long kernel_launches;          /* kernels this context launched                 */
    long long eig_sweeps;               /* implicit QR sweeps, summed over matrices       */
    long long frame_steps;              /* frame-steps processed by cir_run*              */
    double    ms_build, ms_eig, ms_prop, ms_tcf;   /* device time per stage of cir_run*  */
    double    ms_tridiag;               /* of ms_eig: the tridiagonalisation kernel       */
    long long eig_matrices;             /* Hamiltonians built and diagonalised by cir_run* */
    int       tuned_split_tile;         /* autotuner (autotune 1): tile width (128 or 256) it chose
                                           for the last tuned tensor-core propagation product, 0 none */
    int       tuned_tridiag_blocks;     /* autotuner: tridiagonalisation blocks per SM it chose for
                                           the last tuned order, 0 none                       */
} cir_stats;

/* Parameters for the seeded synthetic water-box generator (replaces the .xtc source). */
typedef struct cir_synth {
    int      nmol;
    uint64_t seed;
    double   box_nm;        /* cubic box edge; <= 0 means 1.2417*(nmol/64)^(1/3)       */
    double   frame_dt;      /* ps between frames                                        */
    double   sigma_trans;   /* nm, per axis per frame                                   */
    double   sigma_rot_deg; /* rotation angle per frame                                 */
    double   jitter;        /* nm, lattice jitter of the first frame                    */
    double   min_contact;   /* nm, smallest allowed O/H distance between two molecules  */
    int      max_tries;     /* redraws of one move before the molecule keeps its place  */
} cir_synth;

typedef struct cir_ctx cir_ctx;

/* ---------------- library ---------------- */
const char *cir_version(void);
const char *cir_last_error(void);            /* thread-local message of the last error */

/* ---------------- parameters and files (host only) ---------------- */
int cir_params_default(cir_params *p);                          /* calcIR.cu:36-59      */
int cir_params_parse_file(const char *path, cir_params *p);     /* ir_init calcIR.cu:1539-1643 */
int cir_params_finalize(cir_params *p);                         /* calcIR.cu:94, 324-339 */
int cir_nomega(const cir_params *p);                            /* calcIR.cu:94          */
int cir_result_sizes(const cir_params *p, int *ntcf, int *nomega, int *nls); /* calcIR.cu:890-919 */
int cir_frame_index(const cir_params *p, float frame_dt, int sample, int step, int *frame); /* calcIR.cu:378-379 */
int cir_write_outputs(const cir_params *p, const cir_result *r); /* calcIR.cu:843-919    */

int cir_synth_default(cir_synth *s, int nmol);
/* frames 0..nframes-1 of the trajectory: xyz [nframes][4*nmol][3] (O,H1,H2,M), box [3] */
int cir_synth_trajectory(const cir_synth *s, int nframes, float *xyz, float *box,
                         long long *n_rejected);                /* replaces xtc reading calcIR.cu:376-398 */

/* raw trajectory files ("CIRTRJ01"): header, then per frame time, box[3], xyz[natoms][3] */
int cir_traj_write(const char *path, int natoms, int nframes, float frame_dt,
                   const float *times, const float *boxes, const float *xyz);
int cir_traj_info(const char *path, int *natoms, int *nframes, float *frame_dt); /* read_xtc_natoms calcIR.cu:212 */
int cir_traj_read(const char *path, int first, int count, float *xyz, float *boxes,
                  float *times);

/* Writes a GROMACS .xtc trajectory (XDR, compressed coordinates at `precision` per nm, e.g.
 * 1000): boxes [nframes][3] (diagonal), times [nframes] ps (NULL: 0).  cir_traj_info and
 * cir_traj_read read .xtc files as well as CIRTRJ01 ones, so the drop-in executable takes
 * `xtcf traj.xtc` like the reference (which reads through libxdrfile, calcIR.cu:212-223). */
int cir_xtc_write(const char *path, int natoms, int nframes, const float *xyz, const float *boxes,
                  const float *times, float precision);                                /* xdr_seek + read_xtc calcIR.cu:380-390 */

/* ---------------- engine ---------------- */
int cir_create(const cir_params *p, int natoms, cir_ctx **out); /* allocations + magma_init calcIR.cu:230-319 */
int cir_destroy(cir_ctx *c);                                    /* frees calcIR.cu:922-1006 */
int cir_set_stream(cir_ctx *c, void *cuda_stream);              /* NULL = the context's own stream */
int cir_synchronize(cir_ctx *c);
int cir_get_stats(cir_ctx *c, cir_stats *s);
int cir_reset_stats(cir_ctx *c);

/* Field projection at every H, maps, Hamiltonian, dipoles and polarisabilities for
 * nframes frames: xyz [nframes][natoms][3], box [nframes][3]; outputs (any may be NULL
 * except H): H [nframes][N][N] (symmetric), eproj [nframes][N], dip [nframes][3][N]
 * (x,y,z), pol [nframes][6][N] (xx,yy,zz,xy,yz,zx).
 * Replaces get_eproj_GPU + get_kappa_GPU (calcIR.cu:404-406, 1020-1406). */
int cir_build_hamiltonian(cir_ctx *c, int nframes, const float *xyz, const float *box,
                          float *H, float *eproj, float *dip, float *pol);

/* Batched symmetric eigensolver: A [nmat][n][n] symmetric on entry; on return column j
 * (A[m][j][0..n)) holds eigenvector j and w [nmat][n] the eigenvalues in ascending order.
 * Replaces magma_ssyevd_gpu + the w copy (calcIR.cu:420-448). */
int cir_eigh(cir_ctx *c, int nmat, int n, float *A, float *w);

/* The batched eigensolver of cir_eigh for callers that cannot allocate device memory
 * (no counterpart in the reference).  A host application that owns the GPU memory
 * budget -- for example a simulation engine calling this per frame from inside its own
 * time step -- cannot let a library call cudaMalloc/cudaFree, which synchronise the
 * device and can fail mid-run.  This entry point allocates nothing: A [nmat][n][n] and
 * w [nmat][n] are the caller's DEVICE buffers (same meaning as cir_eigh), and all scratch
 * lives in one 8 MiB device array that every GPU which loads the library holds until the
 * process exits.  Requests whose scratch exceeds 8 MiB are rejected with CIR_ERR_ARG:
 * orders above 1412 (above 1006 when n is not a multiple of 4 or A is not 16-byte
 * aligned, since A is then copied into the scratch first), and batches of more than one
 * matrix of order 1024, seven of order 512 or 25 of order 256 per call; split the batch
 * instead.
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress,
 * which also loads the library's device code on that device under lazy module loading);
 * make that first call before any stream capture.  All calls share the one array and
 * every call overwrites it, so calls that overlap on the GPU (different streams or host
 * threads without ordering) race.  The call is synchronous: it is issued on cuda_stream
 * (NULL: the default stream), reads the per-matrix convergence flags back with
 * cudaMemcpyAsync into a host stack buffer and returns after cudaStreamSynchronize. */
int cir_eigh_noalloc(int nmat, int n, float *A, float *w, void *cuda_stream);

/* The two-stage reduction of nmat symmetric matrices A [nmat][n][n] to tridiagonal form
 * (no counterpart in the reference, whose magma_ssyevd_gpu reduces in one stage,
 * calcIR.cu:443-445): dense -> band of width 32 with the two-sided updates on the
 * split-BF16 tensor-core GEMM, then band -> tridiagonal by bulge chasing.  d [nmat][n]
 * receives the diagonal, e [nmat][n] the subdiagonal (e[n-1] = 0); their eigenvalues are
 * A's to the split-BF16 precision (about 2^-16 of the spread of A's spectrum).  No
 * eigenvectors: the reflectors of both stages are not kept.  n from 3 to 1025.  ms, when
 * not NULL, receives the device time of the two stages in milliseconds. */
int cir_tridiag_sbr(cir_ctx *c, int nmat, int n, const float *A, float *d, float *e, float *ms);

/* One propagation step of nprop independent chains: F <- V diag(exp(+i w dt/hbar)) V^T F,
 * V [nprop][n][n] eigenvectors as returned by cir_eigh, w [nprop][n], F [nprop][n][n]
 * complex.  Replaces Pinit + 3 x magma_cgemm + magma_ccopy (calcIR.cu:596-617). */
int cir_propagate(cir_ctx *c, int nprop, int n, const float *V, const float *w, float dt,
                  float *F);

/* Correlation terms of one frame: out[6] = IR, VV, VH (re, im) increments
 * sum mu_a(t) F mu_a(0) and the Raman combinations.
 * dip0/dip [3][n], pol0/pol [6][n], F [n][n] complex.
 * Replaces the 15 magma_cgemv + magma_cdotu pairs (calcIR.cu:628-745). */
int cir_tcf_terms(cir_ctx *c, int n, const float *F, const float *dip0, const float *pol0,
                  const float *dip, const float *pol, double *out);

/* Lorentzian spectral density of one frame added into Sw [nomega]: V, w as from cir_eigh,
 * dip [3][n].  Replaces 3 x magma_sgemv + get_spectral_density (calcIR.cu:458-482, 1414-1444). */
int cir_spectral_density(cir_ctx *c, int n, const float *V, const float *w, const float *dip,
                         float *Sw);

/* Lineshape of a damped TCF [ntcf][2] (re,im): the unnormalised inverse real DFT of the
 * zero-padded TCF (hand-written mixed-radix FFT), mapped to descending frequencies in
 * [omegaStart, omegaStop]; writes nls rows.  Replaces cufftExecC2R + the output mapping
 * (calcIR.cu:772-827, 890-919). */
int cir_lineshape(cir_ctx *c, const double *tcf, float *omega, float *intensity, int *nls);

/* The whole job: nframes distinct frames xyz [nframes][natoms][3], box [nframes][3];
 * frame_of_step [nsamples*ntcfpoints] picks the frame of every (sample, step) (NULL: the
 * identity, nframes == nsamples*ntcfpoints).  Fills every output array of r.
 * Replaces the sample/frame loops and the finishing steps of main (calcIR.cu:360-839). */
int cir_run(cir_ctx *c, int nframes, const float *xyz, const float *box,
            const int *frame_of_step, cir_result *r);

/* Differentiation form.  The 13 map and coupling coefficients of calcIR.cu:1207-1242 in the
 * order w0 w1 w2 (frequency map), x0 x1 (position matrix element, which also scales the
 * polarisabilities), p0 p1 (momentum), mup0 mup1 mup2 (dipole derivative), wi0 wi1 wi2
 * (intramolecular coupling).  cir_set_coeffs replaces the context's coefficients for every
 * later call (targets, finite differences, fits). */
#define CIR_NTHETA 13
int cir_get_coeffs(cir_ctx *c, float *theta);
int cir_set_coeffs(cir_ctx *c, const float *theta);

/* The backward entry: L = sum over the printed lineshape rows of (IR - target_ir)^2 +
 * (VV - target_vv)^2 for the job cir_run would compute on these frames, and dL/dtheta
 * (grad [CIR_NTHETA], double).  The adjoint runs through the propagation (psi_c = F m_c(0),
 * checkpointed every 16 steps and recomputed in the backward pass) and the eigendecompositions
 * (the Daleckii-Krein divided difference of exp(i L dt/hbar), finite for equal eigenvalues),
 * then through the maps.  FP32 with FP64 sums; nls must equal the lineshape's row count.
 * Extends cir_run (calcIR.cu:360-839); the reference has no gradient. */
int cir_loss_grad(cir_ctx *c, int nframes, const float *xyz, const float *box, const int *frame_of_step,
                  const float *target_ir, const float *target_vv, int nls, double *loss, double *grad);

/* One trajectory of a multi-trajectory job. */
typedef struct cir_traj_in {
    int          natoms;          /* its own system size (a multiple of natom_mol)           */
    int          nframes;
    const float *xyz;             /* [nframes][natoms][3] nm, host or device                  */
    const float *box;             /* [nframes][3]                                             */
    const int   *frame_of_step;   /* [nsamples*ntcfpoints], or NULL for the identity           */
} cir_traj_in;

/* Many independent trajectories, boxes of uneven size allowed, with the context's
 * parameters (its own natoms is not used): trajectories of equal size are batched through
 * every launch (their eigensolves, propagation steps and contractions share launches), the
 * per-step launches are replayed from captured CUDA graphs (cuda_graphs) and the SIMT GEMM
 * tile shapes come from the autotuner (autotune).  results[i] receives trajectory i's
 * outputs exactly as cir_run would fill them.  No counterpart in the reference, which runs
 * one trajectory per process (calcIR.cu:360-839 per run). */
int cir_run_multi(cir_ctx *c, int ntraj, const cir_traj_in *traj, cir_result *results);

#ifdef __cplusplus
}
#endif
#endif /* CALCIR_H_ */
