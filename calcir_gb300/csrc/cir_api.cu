// C ABI of the engine: context, stage entry points and the whole-job driver cir_run.
//
// cir_run processes the nsamples x ntcfpoints frame-steps of a job in chunks of
// consecutive steps for all time origins at once:
//   1. gather the chunk's frames, build every Hamiltonian (one launch pair),
//   2. diagonalise all of them (one batched launch; the frequency distribution of every
//      eigenvector is binned in the same kernel),
//   3. at step 0 of every origin: spectral density,
//   4. for each step: propagate the F of every origin (two batched GEMMs) and contract
//      the correlation terms (one launch).
// The reference runs the same steps frame by frame with host round trips in between
// (calcIR.cu:360-760): the eigenvalues come back to the host from ssyevd, the
// eigenvectors are copied to the host every frame for the frequency distribution, and
// every one of the 15 correlation dot products returns a scalar to the host.  Here
// nothing leaves the device until the job ends.
#include "cir_device.cuh"
#include "cir_plan.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <tuple>
#include <algorithm>
#include <vector>

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

enum {
    B_IN0, B_IN1, B_IN2, B_IN3, B_IN4, B_IN5,      // staging of host arguments
    B_CT, B_Z, B_STATUS, B_SCR,                    // stage scratch
    B_XYZ, B_BOX, B_FIDX, B_CXYZ, B_CBOX,          // run: frames and their gather
    B_A, B_W, B_M, B_F, B_G, B_M0,                 // run: matrices
    B_TCF, B_HCNT, B_HIPR, B_HMIPR, B_OOR, B_SW, B_MU2, B_SWEEPS, B_ROT, B_PAD,
    B_FFT0, B_FFT1, B_FFTY, B_FFTX, B_PROF, B_DE, B_ERR, B_DC, B_TUNE,
    B_PSI, B_LAM, B_PA, B_PB, B_SEG, B_CKPT, B_R, B_T, B_GRAD,   // differentiation form
    B_VS, B_FS,                                    // split-BF16 propagation operands
    B_UFR,                                         // run: distinct frames of a chunk and their multiplicity
    B_HREF, B_RW,                                  // FP64 eigenpair refinement: input copy, workspace
    B_TQW,                                         // the panels' W of a joint tridiagonalisation
    B_COUNT
};

}  // namespace

// A captured step loop: its launch parameters (shapes, pointers, step range) and executable.
struct GraphEntry {
    std::vector<long long> key;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
};

using GemmShape = std::tuple<int, int, int, int, bool, int>;   // M, N, K, batch, A column-major, epilogue

struct cir_ctx {
    cir_params p;
    int natoms = 0, nmol = 0, n = 0, ld = 0;
    int device = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    cudaStream_t aux = nullptr;   // the second half of a split eigensolver batch
    cudaEvent_t xev[3] = {};      // fork, its tridiagonalisation done, join
    DevBuf buf[B_COUNT];
    cir_stats stats;
    cudaEvent_t ev[8];
    CirMaps maps;
    std::map<GemmShape, int> gemm_tile;   // autotuner: SIMT tile shape per product shape
    // autotuner, mixed forms: tile width of each split-BF16 product shape (M, N, K, batch,
    // epilogue, output form, fused contraction) and tridiagonalisation blocks per SM per order
    std::map<std::tuple<int, int, int, int, int, int, int>, int> split_tile;
    std::map<int, int> tq_blocks;
    int last_split_tile = 0, last_tq_blocks = 0;
    std::vector<GraphEntry> graphs;       // captured step loops, most recent last
    // device buffers of the second and later groups of a joint cir_run_multi job
    std::vector<std::unique_ptr<DevBuf[]>> gbuf;
};

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

static bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// CIR_EIGH_PROFILE=1: per-phase wall time of the eigensolver blocks, printed to stderr
static bool eigh_profiling() {
    const char *v = getenv("CIR_EIGH_PROFILE");
    return v && v[0] == '1';
}

static void eigh_profile_report(const unsigned long long *dev, int nmat, cudaStream_t s) {
    const int S = CIR_EIG_PROF_SLOTS;
    std::vector<unsigned long long> h((size_t)nmat * S);
    if (cudaMemcpyAsync(h.data(), dev, h.size() * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess) return;
    cudaStreamSynchronize(s);
    double tri = 0, fq = 0, qr = 0, srt = 0, chase = 0, apply = 0, nrot = 0, search = 0, sweeps = 0;
    double tqp[6] = {0, 0, 0, 0, 0, 0};
    unsigned long long t0 = ~0ull, t1 = 0;
    for (int m = 0; m < nmat; m++) {
        const unsigned long long *r = h.data() + (size_t)m * S;
        tri += (double)(r[1] - r[0]);
        fq += (double)(r[3] - r[2]);
        qr += (double)(r[5] - r[4]);
        srt += (double)(r[6] - r[5]);
        t0 = std::min(t0, r[0]);
        t1 = std::max(t1, r[1]);
        chase += (double)r[7];
        apply += (double)r[8];
        nrot += (double)r[9];
        search += (double)r[10];
        sweeps += (double)r[11];
        for (int q = 0; q < 6; q++) tqp[q] += (double)r[12 + q];
    }
    fprintf(stderr, "eigh profile: %d matrices, tridiagonalisation span %.3f ms; mean per block (ms): tridiag %.3f formQ %.3f qr %.3f "
                    "(chase %.3f incl. block search %.3f, apply %.3f, %.0f rotations in %.0f sweeps) sort %.3f\n",
            nmat, (t1 - t0) * 1e-6, tri / nmat * 1e-6, fq / nmat * 1e-6, qr / nmat * 1e-6, chase / nmat * 1e-6,
            search / nmat * 1e-6, apply / nmat * 1e-6, nrot / nmat, sweeps / nmat, srt / nmat * 1e-6);
    double mp[5] = {0, 0, 0, 0, 0};
    for (int m = 0; m < nmat; m++)
        for (int q = 0; q < 5; q++) mp[q] += (double)h[(size_t)m * S + 7 + q];
    double itn = 0, rts = 0;
    for (int m = 0; m < nmat; m++) { itn += (double)h[(size_t)m * S + 18]; rts += (double)h[(size_t)m * S + 19]; }
    if (rts > 0) fprintf(stderr, "eigh profile: secular equation: %.2f iterations per root over %.0f roots\n", itn / rts, rts);
    if (mp[1] > 0)
        fprintf(stderr, "eigh profile: merges, summed over a matrix's merges, mean per matrix (ms): setup and deflation "
                        "%.3f roots %.3f z and norms %.3f ranking %.3f rotation %.3f\n",
                mp[0] / nmat * 1e-6, mp[1] / nmat * 1e-6, mp[2] / nmat * 1e-6, mp[3] / nmat * 1e-6, mp[4] / nmat * 1e-6);
    if (tqp[0] + tqp[2] > 0)
        fprintf(stderr, "eigh profile: tridiagonalisation phases, mean per block (ms): column %.3f reflector %.3f "
                        "symv %.3f panel dots %.3f w %.3f trailing update %.3f\n",
                tqp[0] / nmat * 1e-6, tqp[1] / nmat * 1e-6, tqp[2] / nmat * 1e-6, tqp[3] / nmat * 1e-6,
                tqp[4] / nmat * 1e-6, tqp[5] / nmat * 1e-6);
}

static int count_launch(cir_ctx *c, int k) {
    c->stats.kernel_launches += k;
    return CIR_OK;
}

// Device pointer for an argument: the pointer itself, or a staging buffer filled from host.
static int stage_in(cir_ctx *c, int slot, const void *host_or_dev, size_t bytes, void **out, bool copy) {
    if (is_device_ptr(host_or_dev)) {
        *out = const_cast<void *>(host_or_dev);
        return CIR_OK;
    }
    CK(c->buf[slot].ensure(bytes));
    if (copy && host_or_dev) CK(cudaMemcpyAsync(c->buf[slot].p, host_or_dev, bytes, cudaMemcpyHostToDevice, c->stream));
    *out = c->buf[slot].p;
    return CIR_OK;
}

static int stage_out(cir_ctx *c, void *dst, const void *dev, size_t bytes) {
    if (!dst || dst == dev) return CIR_OK;
    CK(cudaMemcpyAsync(dst, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    return CIR_OK;
}

// Compensated (Neumaier) FP64 sum: the running error term keeps what each addition rounds
// away, so a long sum over time origins (hundreds of terms of either sign, partly
// cancelling at long times) carries an error of O(eps) instead of O(S eps).
struct CompSum {
    double s = 0.0, e = 0.0;
    void add(double x) {
        const double t = s + x;
        e += std::fabs(s) >= std::fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    double value() const { return s + e; }
};

static bool all_finite(const float *x, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!std::isfinite(x[i])) return false;
    return true;
}

extern "C" int cir_create(const cir_params *p, int natoms, cir_ctx **out) {
    if (!p || !out) return cir_fail(CIR_ERR_ARG, "cir_create: null pointer");
    *out = nullptr;
    cir_params q = *p;
    int rc = cir_params_finalize(&q);
    if (rc) return rc;
    if (natoms < q.natom_mol || natoms % q.natom_mol)
        return cir_fail(CIR_ERR_ARG, "natoms %d is not a positive multiple of natom_mol %d", natoms, q.natom_mol);

    const int nmol = natoms / q.natom_mol;
    const int n = nmol * q.nchrom_mol;
    if (n > cir_eigh_max_n()) return cir_fail(CIR_ERR_ARG, "%d chromophores exceed the supported %d", n, cir_eigh_max_n());
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return cir_fail(CIR_ERR_NODEVICE, "no CUDA device is available");
    }
    cir_ctx *c = new cir_ctx();
    c->p = q;
    c->natoms = natoms;
    c->nmol = nmol;
    c->n = n;
    c->ld = (n + 3) & ~3;
    cir_maps(q.map, q.ispecies, &c->maps);
    memset(&c->stats, 0, sizeof c->stats);
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    for (int i = 0; e == cudaSuccess && i < 8; i++) e = cudaEventCreate(&c->ev[i]);
    if (e != cudaSuccess) {
        delete c;
        return cir_fail(CIR_ERR_CUDA, "cir_create: %s", cudaGetErrorString(e));
    }
    c->stream = c->own;
    if (c->buf[B_ERR].ensure(sizeof(int)) != cudaSuccess || cudaMemset(c->buf[B_ERR].p, 0, sizeof(int)) != cudaSuccess) {
        cir_destroy(c);
        return cir_fail(CIR_ERR_CUDA, "cir_create: cannot allocate the error flag");
    }
    *out = c;
    return CIR_OK;
}

// The tensor-core kernels set the context's error flag when a bounded wait gives up.
static int check_kernel_flag(cir_ctx *c) {
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, c->buf[B_ERR].p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (flag) {
        cudaMemsetAsync(c->buf[B_ERR].p, 0, sizeof(int), c->stream);
        return cir_fail(CIR_ERR_CUDA, "a tensor-core kernel timed out waiting on its pipeline");
    }
    return CIR_OK;
}

extern "C" int cir_destroy(cir_ctx *c) {
    if (!c) return CIR_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    for (auto &b : c->buf) b.release();
    for (auto &gb : c->gbuf)
        for (int i = 0; i < B_COUNT; i++) gb[i].release();
    for (auto &e : c->ev) cudaEventDestroy(e);
    for (auto &e : c->xev)
        if (e) cudaEventDestroy(e);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return CIR_OK;
}

extern "C" int cir_set_stream(cir_ctx *c, void *s) {
    if (!c) return cir_fail(CIR_ERR_ARG, "cir_set_stream: null context");
    c->stream = s ? static_cast<cudaStream_t>(s) : c->own;
    return CIR_OK;
}

extern "C" int cir_synchronize(cir_ctx *c) {
    if (!c) return cir_fail(CIR_ERR_ARG, "cir_synchronize: null context");
    CK(cudaStreamSynchronize(c->stream));
    return CIR_OK;
}

extern "C" int cir_get_stats(cir_ctx *c, cir_stats *s) {
    if (!c || !s) return cir_fail(CIR_ERR_ARG, "cir_get_stats: null pointer");
    *s = c->stats;
    s->tuned_split_tile = c->last_split_tile;
    s->tuned_tridiag_blocks = c->last_tq_blocks;
    return CIR_OK;
}

extern "C" int cir_reset_stats(cir_ctx *c) {
    if (!c) return cir_fail(CIR_ERR_ARG, "cir_reset_stats: null context");
    memset(&c->stats, 0, sizeof c->stats);
    return CIR_OK;
}

// One group of a run: ntraj trajectories of one system size, batched through every launch.
struct Group {
    int natoms, nmol, n, ld, ntraj;
};

static Group ctx_group(const cir_ctx *c) { return Group{c->natoms, c->nmol, c->n, c->ld, 1}; }

static BuildArgs build_args(cir_ctx *c, const Group &g) {
    BuildArgs a;
    memset(&a, 0, sizeof a);
    a.natoms = g.natoms;
    a.natom_mol = c->p.natom_mol;
    a.nchrom_mol = c->p.nchrom_mol;
    a.nmol = g.nmol;
    a.n = g.n;
    a.ld = g.ld;
    a.imodel = c->p.imodel;
    a.ispecies = c->p.ispecies;
    a.avef = c->p.avef;
    a.maps = c->maps;
    return a;
}

extern "C" int cir_build_hamiltonian(cir_ctx *c, int nframes, const float *xyz, const float *box, float *H,
                                     float *eproj, float *dip, float *pol) {
    if (!c || !xyz || !box || !H || nframes < 1) return cir_fail(CIR_ERR_ARG, "cir_build_hamiltonian: bad argument");
    const int n = c->n;
    const size_t nx = (size_t)nframes * c->natoms * 3;
    if (!is_device_ptr(xyz) && !all_finite(xyz, nx)) return cir_fail(CIR_ERR_NONFINITE, "positions contain NaN or Inf");
    if (!is_device_ptr(box) && !all_finite(box, 3 * (size_t)nframes)) return cir_fail(CIR_ERR_NONFINITE, "box contains NaN or Inf");
    void *dx, *db, *dH, *dE = nullptr, *dD = nullptr, *dP = nullptr;
    int rc;
    if ((rc = stage_in(c, B_IN0, xyz, nx * 4, &dx, true))) return rc;
    if ((rc = stage_in(c, B_IN1, box, (size_t)nframes * 12, &db, true))) return rc;
    if ((rc = stage_in(c, B_IN2, H, (size_t)nframes * n * n * 4, &dH, false))) return rc;
    if (eproj && (rc = stage_in(c, B_IN3, eproj, (size_t)nframes * n * 4, &dE, false))) return rc;
    if (dip && (rc = stage_in(c, B_IN4, dip, (size_t)nframes * 3 * n * 4, &dD, false))) return rc;
    if (pol && (rc = stage_in(c, B_IN5, pol, (size_t)nframes * 6 * n * 4, &dP, false))) return rc;
    CK(c->buf[B_CT].ensure((size_t)nframes * CT_NROW * c->ld * 4));
    BuildArgs a = build_args(c, ctx_group(c));
    a.xyz = static_cast<const float *>(dx);
    a.box = static_cast<const float *>(db);
    a.ct = c->buf[B_CT].as<float>();
    a.H = static_cast<float *>(dH);
    a.ldh = n;
    a.eproj = static_cast<float *>(dE);
    a.dip = static_cast<float *>(dD);
    a.pol = static_cast<float *>(dP);
    a.ldv = n;
    a.dip_fstride = 3LL * n;
    a.pol_fstride = 6LL * n;
    int launches = 0;
    CK(cir_launch_build(a, nframes, c->stream, &launches));
    count_launch(c, launches);
    if ((rc = stage_out(c, H, dH, (size_t)nframes * n * n * 4))) return rc;
    if (eproj && (rc = stage_out(c, eproj, dE, (size_t)nframes * n * 4))) return rc;
    if (dip && (rc = stage_out(c, dip, dD, (size_t)nframes * 3 * n * 4))) return rc;
    if (pol && (rc = stage_out(c, pol, dP, (size_t)nframes * 6 * n * 4))) return rc;
    if (!is_device_ptr(H)) CK(cudaStreamSynchronize(c->stream));
    return CIR_OK;
}

static int setup_refine(cir_ctx *c, EighArgs &e, int nmat);

extern "C" int cir_eigh(cir_ctx *c, int nmat, int n, float *A, float *w) {
    if (!c || !A || !w || nmat < 1 || n < 1) return cir_fail(CIR_ERR_ARG, "cir_eigh: bad argument");
    if (n > cir_eigh_max_n()) return cir_fail(CIR_ERR_ARG, "cir_eigh: n = %d exceeds %d", n, cir_eigh_max_n());
    if (nmat > 65535) return cir_fail(CIR_ERR_ARG, "cir_eigh: %d matrices in one call (at most 65535)", nmat);
    if (!is_device_ptr(A) && !all_finite(A, (size_t)nmat * n * n))
        return cir_fail(CIR_ERR_NONFINITE, "cir_eigh: the matrices contain NaN or Inf");
    // the kernel wants a leading dimension that is a multiple of 4: stage through a padded copy
    const int ld = (n + 3) & ~3;
    const size_t mb = (size_t)n * ld * 4;
    CK(c->buf[B_PAD].ensure(nmat * mb));
    CK(c->buf[B_Z].ensure(nmat * mb));
    CK(c->buf[B_DC].ensure(nmat * cir_dc_bytes(n, ld)));
    CK(c->buf[B_DE].ensure(nmat * cir_eigh_de_bytes(ld)));
    CK(c->buf[B_STATUS].ensure((size_t)nmat * 4));
    CK(c->buf[B_SWEEPS].ensure(8));
    CK(c->buf[B_IN1].ensure((size_t)nmat * n * 4));
    CK(cudaMemsetAsync(c->buf[B_SWEEPS].p, 0, 8, c->stream));
    CK(cudaMemcpy2DAsync(c->buf[B_PAD].p, (size_t)ld * 4, A, (size_t)n * 4, (size_t)n * 4, (size_t)nmat * n,
                         cudaMemcpyDefault, c->stream));
    EighArgs a;
    memset(&a, 0, sizeof a);
    a.A = c->buf[B_PAD].as<float>();
    a.W = c->buf[B_IN1].as<float>();
    a.Z = c->buf[B_Z].as<float>();
    a.DC = c->buf[B_DC].as<float>();
    a.DE = c->buf[B_DE].as<float>();
    a.mstride = (long long)n * ld;
    a.wstride = n;
    a.n = n;
    a.ld = ld;
    a.status = c->buf[B_STATUS].as<int>();
    a.sweeps = c->buf[B_SWEEPS].as<unsigned long long>();
    a.nchrom_mol = c->p.nchrom_mol;
    // the mixed forms run the eigensolver's products on the tensor cores as split BF16, as
    // the whole-job path does
    a.precision = c->p.precision == CIR_PREC_FP32 ? CIR_PREC_FP32 : CIR_PREC_BF16X3;
    a.err = c->buf[B_ERR].as<int>();
    a.test_stall = c->p.test_stall_gemm;
    a.test_sweep_cap = c->p.test_sweep_cap;
    if (eigh_profiling()) {
        CK(c->buf[B_PROF].ensure((size_t)nmat * CIR_EIG_PROF_SLOTS * 8));
        CK(cudaMemsetAsync(c->buf[B_PROF].p, 0, (size_t)nmat * CIR_EIG_PROF_SLOTS * 8, c->stream));
        a.phase_ns = c->buf[B_PROF].as<unsigned long long>();
    }
    int rc;
    if ((rc = setup_refine(c, a, nmat))) return rc;
    int launches = 0;
    CK(cir_launch_eigh(a, nmat, c->stream, &launches));
    count_launch(c, launches);
    if (a.phase_ns) eigh_profile_report(a.phase_ns, nmat, c->stream);
    CK(cudaMemcpy2DAsync(A, (size_t)n * 4, c->buf[B_PAD].p, (size_t)ld * 4, (size_t)n * 4, (size_t)nmat * n,
                         cudaMemcpyDefault, c->stream));
    CK(cudaMemcpyAsync(w, a.W, (size_t)nmat * n * 4, cudaMemcpyDefault, c->stream));
    std::vector<int> st(nmat);
    unsigned long long sweeps = 0;
    CK(cudaMemcpyAsync(st.data(), a.status, (size_t)nmat * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&sweeps, a.sweeps, 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->stats.eig_sweeps += (long long)sweeps;
    for (int i = 0; i < nmat; i++)
        if (st[i]) return cir_fail(CIR_ERR_NOCONVERGE, "eigensolver sweep cap reached on matrix %d", i);
    if (a.precision != CIR_PREC_FP32 && (rc = check_kernel_flag(c))) return rc;
    return CIR_OK;
}

extern "C" int cir_tridiag_sbr(cir_ctx *c, int nmat, int n, const float *A, float *d, float *e, float *ms) {
    if (!c || !A || !d || !e || nmat < 1 || n < 3) return cir_fail(CIR_ERR_ARG, "cir_tridiag_sbr: bad argument");
    if (n > cir_sbr_max_n())
        return cir_fail(CIR_ERR_ARG, "cir_tridiag_sbr: n = %d exceeds %d", n, cir_sbr_max_n());
    if (nmat > 65535) return cir_fail(CIR_ERR_ARG, "cir_tridiag_sbr: %d matrices in one call (at most 65535)", nmat);
    if (!is_device_ptr(A) && !all_finite(A, (size_t)nmat * n * n))
        return cir_fail(CIR_ERR_NONFINITE, "cir_tridiag_sbr: the matrices contain NaN or Inf");
    const int ld = (n + 7) & ~7;   // the pairs' rows start on 16-byte boundaries
    CK(c->buf[B_PAD].ensure((size_t)nmat * n * ld * 4));
    CK(c->buf[B_Z].ensure((size_t)nmat * cir_sbr_bytes(n, ld)));
    CK(c->buf[B_IN1].ensure((size_t)nmat * n * 8));
    CK(cudaMemcpy2DAsync(c->buf[B_PAD].p, (size_t)ld * 4, A, (size_t)n * 4, (size_t)n * 4, (size_t)nmat * n,
                         cudaMemcpyDefault, c->stream));
    float *dd = c->buf[B_IN1].as<float>(), *ee = dd + (size_t)nmat * n;
    int launches = 0;
    CK(cir_launch_sbr(c->buf[B_PAD].as<float>(), (long long)n * ld, nmat, n, ld, dd, ee, c->buf[B_Z].p,
                      c->buf[B_ERR].as<int>(), c->stream, ms, &launches));
    count_launch(c, launches);
    CK(cudaMemcpyAsync(d, dd, (size_t)nmat * n * 4, cudaMemcpyDefault, c->stream));
    CK(cudaMemcpyAsync(e, ee, (size_t)nmat * n * 4, cudaMemcpyDefault, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return check_kernel_flag(c);
}

// The optional FP64 refinement of the eigenpairs (refine_eigen steps): a copy of the nmat
// input matrices at e.A, taken before the eigensolver overwrites them, and the workspace for
// as many matrices at a time as fit in 2 GiB.
static int setup_refine(cir_ctx *c, EighArgs &e, int nmat) {
    if (c->p.refine_eigen <= 0) return CIR_OK;
    const size_t mb = (size_t)e.mstride * 4;
    CK(c->buf[B_HREF].ensure(nmat * mb));
    CK(cudaMemcpyAsync(c->buf[B_HREF].p, e.A, nmat * mb, cudaMemcpyDeviceToDevice, c->stream));
    const size_t per = cir_refine_bytes(e.n, e.ld);
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nmat, ((size_t)2 << 30) / per));
    CK(c->buf[B_RW].ensure(chunk * per));
    e.Href = c->buf[B_HREF].as<float>();
    e.RW = c->buf[B_RW].p;
    e.refine_iters = c->p.refine_eigen;
    e.refine_chunk = chunk;
    return CIR_OK;
}

static GemmShape gemm_shape(const GemmArgs &g, int batch) {
    return GemmShape(g.M, g.N, g.K, batch, g.a_colmajor, g.epilogue);
}

// The SIMT tile shape the autotuner chose for this product shape (128 x 128 if untuned).
static int tuned_tile(cir_ctx *c, const GemmArgs &g, int batch) {
    auto it = c->gemm_tile.find(gemm_shape(g, batch));
    return it == c->gemm_tile.end() ? CIR_GEMM_TILE_128 : it->second;
}

// Autotuner: times both SIMT tile shapes of a product shape once per context (on scratch
// operands of the same sizes, so the caller's data is untouched) and keeps the faster.
// Must run outside stream capture.
static int autotune_gemm(cir_ctx *c, const GemmArgs &g, int batch) {
    if (!c->p.autotune || c->gemm_tile.count(gemm_shape(g, batch))) return CIR_OK;
    const size_t a_el = (size_t)(g.a_colmajor ? g.K : g.M) * g.lda, b_el = (size_t)(g.b_kmajor ? g.N : g.K) * g.ldb,
                 c_el = (size_t)g.M * g.ldc, w_el = g.epilogue == 1 ? (size_t)g.M : 0;
    const size_t tot = (a_el + b_el + c_el + w_el + 16) * batch * sizeof(float);
    CK(c->buf[B_TUNE].ensure(tot));
    CK(cudaMemsetAsync(c->buf[B_TUNE].p, 0, tot, c->stream));
    float *base = c->buf[B_TUNE].as<float>();
    GemmArgs t = g;
    t.A = base;
    t.sA = (long long)a_el;
    t.B = base + a_el * batch;
    t.sB = (long long)b_el;
    t.C = base + (a_el + b_el) * batch;
    t.sC = (long long)c_el;
    if (g.epilogue == 1) {
        t.w = base + (a_el + b_el + c_el) * batch;
        t.wstride = g.M;
    }
    float best = 1e30f;
    int pick = CIR_GEMM_TILE_128;
    for (int tile : {CIR_GEMM_TILE_128, CIR_GEMM_TILE_64}) {
        CK(cir_launch_gemm(t, batch, c->stream, nullptr, tile));   // warm-up
        CK(cudaEventRecord(c->ev[6], c->stream));
        for (int r = 0; r < 3; r++) CK(cir_launch_gemm(t, batch, c->stream, nullptr, tile));
        CK(cudaEventRecord(c->ev[7], c->stream));
        CK(cudaEventSynchronize(c->ev[7]));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]));
        if (ms < best) { best = ms; pick = tile; }
    }
    c->gemm_tile[gemm_shape(g, batch)] = pick;
    if (c->p.verbose) printf("autotune: GEMM %d x %d x %d (batch %d): %s tiles\n", g.M, g.N, g.K, batch,
                             pick == CIR_GEMM_TILE_64 ? "64 x 64" : "128 x 128");
    return CIR_OK;
}

static std::tuple<int, int, int, int, int, int, int> split_shape(const SplitGemmArgs &g, int batch) {
    return std::make_tuple(g.M, g.N, g.K, batch, g.epilogue, g.out_mode, g.tcf_out != nullptr ? 1 : 0);
}

// The tile width the autotuner chose for a split-BF16 product shape (0: the launcher's own).
static int tuned_split(cir_ctx *c, const SplitGemmArgs &g, int batch) {
    auto it = c->split_tile.find(split_shape(g, batch));
    return it == c->split_tile.end() ? 0 : it->second;
}

// Autotuner for the tensor-core form: times the persistent split-BF16 GEMM with 128 x 128
// and 128 x 256 tiles once per product shape, on zeroed scratch operands of the same sizes
// and strides (the caller's data untouched; the fused contraction's sums go to scratch),
// and keeps the faster.  Both widths accumulate every output in the same order, so the
// choice changes speed only.  Must run outside stream capture.
static int autotune_split(cir_ctx *c, const SplitGemmArgs &g, int batch) {
    if (!c->p.autotune || c->split_tile.count(split_shape(g, batch))) return CIR_OK;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t a_b = al((size_t)g.sA * batch * 2), b_b = al((size_t)g.sB * batch * 2),
                 c_b = al((size_t)g.sC * batch * (g.out_mode == 2 ? 4 : 2)), d_b = g.epilogue == 2 ? al((size_t)g.sD * batch * 2) : 0,
                 w_b = g.epilogue == 1 ? al((size_t)g.wstride * batch * 4 + 64) : 0,
                 m_b = g.tcf_out ? al(((size_t)g.tcf_sm0 + g.tcf_smt) * batch * 4 + 64) : 0,
                 o_b = g.tcf_out ? al((size_t)g.tcf_sout * batch * 8 + 64) : 0;
    const size_t tot = 2 * a_b + 2 * b_b + 2 * c_b + 2 * d_b + w_b + m_b + o_b;
    CK(c->buf[B_TUNE].ensure(tot));
    CK(cudaMemsetAsync(c->buf[B_TUNE].p, 0, tot, c->stream));
    unsigned char *q = c->buf[B_TUNE].as<unsigned char>();
    auto take = [&](size_t b) { unsigned char *r = q; q += b; return r; };
    SplitGemmArgs t = g;
    t.Ahi = reinterpret_cast<__nv_bfloat16 *>(take(a_b)); t.Alo = reinterpret_cast<__nv_bfloat16 *>(take(a_b));
    t.Bhi = reinterpret_cast<__nv_bfloat16 *>(take(b_b)); t.Blo = reinterpret_cast<__nv_bfloat16 *>(take(b_b));
    unsigned char *c0 = take(c_b), *c1 = take(c_b);
    t.Chi = reinterpret_cast<__nv_bfloat16 *>(c0); t.Clo = reinterpret_cast<__nv_bfloat16 *>(c1);
    t.Cf = reinterpret_cast<float *>(c0);
    if (d_b) { t.Dhi = reinterpret_cast<__nv_bfloat16 *>(take(d_b)); t.Dlo = reinterpret_cast<__nv_bfloat16 *>(take(d_b)); }
    if (w_b) t.w = reinterpret_cast<float *>(take(w_b));
    if (m_b) {
        float *m = reinterpret_cast<float *>(take(m_b));
        t.tcf_m0 = m;
        t.tcf_mt = m + (size_t)g.tcf_sm0 * batch;
    }
    if (o_b) t.tcf_out = reinterpret_cast<double *>(take(o_b));
    t.test_stall = 0;
    float best = 1e30f;
    int pick = 0;
    for (int tile : {128, 256}) {
        t.tile_n = tile;
        CK(cir_launch_split_gemm(t, batch, c->stream, nullptr));   // warm-up
        CK(cudaEventRecord(c->ev[6], c->stream));
        for (int r = 0; r < 3; r++) CK(cir_launch_split_gemm(t, batch, c->stream, nullptr));
        CK(cudaEventRecord(c->ev[7], c->stream));
        CK(cudaEventSynchronize(c->ev[7]));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]));
        if (ms < best) { best = ms; pick = tile; }
    }
    c->buf[B_TUNE].release();
    c->split_tile[split_shape(g, batch)] = pick;
    c->last_split_tile = pick;
    if (c->p.verbose) printf("autotune: split-BF16 GEMM %d x %d x %d (batch %d): 128 x %d tiles\n", g.M, g.N, g.K,
                             batch, pick);
    return CIR_OK;
}

// Autotuner for the tridiagonalisation: blocks per SM (its own occupancy or one less),
// timed once per order on copies of up to 6 waves of the caller's first matrices, restored
// before every trial; keeps the faster per matrix.  Must run outside stream capture.
static int autotune_tridiag(cir_ctx *c, const EighArgs &e, int nmat) {
    if (!c->p.autotune || c->tq_blocks.count(e.n)) return CIR_OK;
    const int def = cir_tridiag_blocks(e.n);
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int sample = std::min(nmat, 6 * sms);
    if (def < 2 || sample < 2 * sms) {   // too few matrices to tell the variants apart
        c->tq_blocks[e.n] = 0;
        return CIR_OK;
    }
    const size_t mb = (size_t)e.mstride * 4;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t a_b = al(sample * mb), de_b = al(sample * cir_eigh_de_bytes(e.ld)), st_b = al((size_t)sample * 4);
    CK(c->buf[B_TUNE].ensure(3 * a_b + de_b + st_b));
    unsigned char *q = c->buf[B_TUNE].as<unsigned char>();
    float *orig = reinterpret_cast<float *>(q), *work = reinterpret_cast<float *>(q + a_b);
    EighArgs t;
    memset(&t, 0, sizeof t);
    t.A = work;
    t.Z = reinterpret_cast<float *>(q + 2 * a_b);
    t.DE = reinterpret_cast<float *>(q + 3 * a_b);
    t.status = reinterpret_cast<int *>(q + 3 * a_b + de_b);
    t.mstride = e.mstride;
    t.n = e.n;
    t.ld = e.ld;
    CK(cudaMemcpyAsync(orig, e.A, sample * mb, cudaMemcpyDeviceToDevice, c->stream));
    float best = 1e30f;
    int pick = 0;
    for (int blocks : {def, def - 1}) {
        t.tq_blocks = blocks;
        float ms_best = 1e30f;
        for (int r = 0; r < 2; r++) {
            CK(cudaMemcpyAsync(work, orig, sample * mb, cudaMemcpyDeviceToDevice, c->stream));
            CK(cudaEventRecord(c->ev[6], c->stream));
            CK(cir_launch_tridiag(t, sample, c->stream));
            CK(cudaEventRecord(c->ev[7], c->stream));
            CK(cudaEventSynchronize(c->ev[7]));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]));
            ms_best = std::min(ms_best, ms);
        }
        if (ms_best < best) { best = ms_best; pick = blocks; }
    }
    c->buf[B_TUNE].release();
    c->tq_blocks[e.n] = pick == def ? 0 : pick;
    c->last_tq_blocks = pick;
    if (c->p.verbose) printf("autotune: tridiagonalisation of order %d: %d blocks per SM\n", e.n, pick);
    return CIR_OK;
}

// F <- V diag(exp(+i w dt/hbar)) V^T F for `nprop` chains; all pointers on the device.
static int propagate_dev(cir_ctx *c, int nprop, int n, const float *V, int ldv, long long sV, const float *w,
                         int wstride, float dt, float *F, int ldf, long long sF, float *G, int &launches) {
    GemmArgs g1;
    memset(&g1, 0, sizeof g1);
    g1.A = V; g1.lda = ldv; g1.sA = sV; g1.a_colmajor = false;      // V^T as a row-major view of V
    g1.B = F; g1.ldb = ldf; g1.sB = sF;
    g1.C = G; g1.ldc = ldf; g1.sC = sF;
    g1.M = n; g1.N = 2 * n; g1.K = n;
    g1.epilogue = 1; g1.w = w; g1.wstride = wstride;
    g1.dt_over_hbar = (float)(dt / CIR_HBAR);
    GemmArgs g2 = g1;
    g2.A = V; g2.a_colmajor = true;                                   // V itself
    g2.B = G; g2.C = F; g2.epilogue = 0;
    if (c->p.precision == CIR_PREC_FP32) {
        CK(cir_launch_gemm(g1, nprop, c->stream, &launches, tuned_tile(c, g1, nprop)));
        CK(cir_launch_gemm(g2, nprop, c->stream, &launches, tuned_tile(c, g2, nprop)));
    } else {
        CK(c->buf[B_ERR].ensure(sizeof(int)));
        g1.err = g2.err = c->buf[B_ERR].as<int>();
        CK(cir_launch_tc_gemm(g1, nprop, c->p.precision, c->stream, &launches));
        CK(cir_launch_tc_gemm(g2, nprop, c->p.precision, c->stream, &launches));
    }
    return CIR_OK;
}

extern "C" int cir_propagate(cir_ctx *c, int nprop, int n, const float *V, const float *w, float dt, float *F) {
    if (!c || !V || !w || !F || nprop < 1 || n < 1) return cir_fail(CIR_ERR_ARG, "cir_propagate: bad argument");
    const size_t mb = (size_t)n * n * 4;
    void *dV, *dW, *dF;
    int rc;
    if ((rc = stage_in(c, B_IN0, V, nprop * mb, &dV, true))) return rc;
    if ((rc = stage_in(c, B_IN1, w, (size_t)nprop * n * 4, &dW, true))) return rc;
    if ((rc = stage_in(c, B_IN2, F, nprop * mb * 2, &dF, true))) return rc;
    CK(c->buf[B_SCR].ensure(nprop * mb * 2));
    int launches = 0;
    rc = propagate_dev(c, nprop, n, static_cast<float *>(dV), n, (long long)n * n, static_cast<float *>(dW), n, dt,
                       static_cast<float *>(dF), 2 * n, 2LL * n * n, c->buf[B_SCR].as<float>(), launches);
    count_launch(c, launches);
    if (rc) return rc;
    if ((rc = stage_out(c, F, dF, nprop * mb * 2))) return rc;
    if (!is_device_ptr(F)) CK(cudaStreamSynchronize(c->stream));
    if (c->p.precision != CIR_PREC_FP32 && (rc = check_kernel_flag(c))) return rc;
    return CIR_OK;
}

extern "C" int cir_tcf_terms(cir_ctx *c, int n, const float *F, const float *dip0, const float *pol0,
                             const float *dip, const float *pol, double *out) {
    if (!c || !F || !dip0 || !pol0 || !dip || !pol || !out || n < 1) return cir_fail(CIR_ERR_ARG, "cir_tcf_terms: bad argument");
    void *dF, *d0, *p0, *d1, *p1;
    int rc;
    if ((rc = stage_in(c, B_IN0, F, (size_t)n * n * 8, &dF, true))) return rc;
    if ((rc = stage_in(c, B_IN1, dip0, (size_t)3 * n * 4, &d0, true))) return rc;
    if ((rc = stage_in(c, B_IN2, pol0, (size_t)6 * n * 4, &p0, true))) return rc;
    if ((rc = stage_in(c, B_IN3, dip, (size_t)3 * n * 4, &d1, true))) return rc;
    if ((rc = stage_in(c, B_IN4, pol, (size_t)6 * n * 4, &p1, true))) return rc;
    CK(c->buf[B_SCR].ensure((size_t)18 * n * 4 + 64));
    float *m = c->buf[B_SCR].as<float>();
    CK(cudaMemcpyAsync(m, d0, (size_t)3 * n * 4, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(m + 3 * n, p0, (size_t)6 * n * 4, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(m + 9 * n, d1, (size_t)3 * n * 4, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(m + 12 * n, p1, (size_t)6 * n * 4, cudaMemcpyDeviceToDevice, c->stream));
    double *acc = reinterpret_cast<double *>(m + 18 * n);
    CK(cudaMemsetAsync(acc, 0, 48, c->stream));
    TcfArgs t;
    memset(&t, 0, sizeof t);
    t.F = static_cast<float *>(dF);
    t.m0 = m;
    t.mt = m + 9 * n;
    t.out = acc;
    t.n = n;
    t.ldf = 2 * n;
    t.ldv = n;
    int launches = 0;
    CK(cir_launch_tcf(t, 1, c->stream, &launches));
    count_launch(c, launches);
    CK(cudaMemcpyAsync(out, acc, 48, is_device_ptr(out) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
    if (!is_device_ptr(out)) CK(cudaStreamSynchronize(c->stream));
    return CIR_OK;
}

extern "C" int cir_spectral_density(cir_ctx *c, int n, const float *V, const float *w, const float *dip, float *Sw) {
    if (!c || !V || !w || !dip || !Sw || n < 1) return cir_fail(CIR_ERR_ARG, "cir_spectral_density: bad argument");
    const int nomega = cir_nomega(&c->p);
    void *dV, *dW, *dD;
    int rc;
    if ((rc = stage_in(c, B_IN0, V, (size_t)n * n * 4, &dV, true))) return rc;
    if ((rc = stage_in(c, B_IN1, w, (size_t)n * 4, &dW, true))) return rc;
    if ((rc = stage_in(c, B_IN2, dip, (size_t)3 * n * 4, &dD, true))) return rc;
    CK(c->buf[B_SCR].ensure((size_t)n * 4 + (size_t)nomega * 8 + 64));
    float *mu2 = c->buf[B_SCR].as<float>();
    double *acc = reinterpret_cast<double *>(c->buf[B_SCR].as<char>() + (((size_t)n * 4 + 15) & ~(size_t)15));
    CK(cudaMemsetAsync(acc, 0, (size_t)nomega * 8, c->stream));
    int launches = 0;
    CK(cir_launch_spectral(static_cast<float *>(dV), n, static_cast<float *>(dW), static_cast<float *>(dD), n, n, mu2,
                           acc, nomega, c->p.omegaStart, c->p.omegaStep, c->p.t1, c->p.avef, c->stream, &launches));
    count_launch(c, launches);
    std::vector<double> h(nomega);
    CK(cudaMemcpyAsync(h.data(), acc, (size_t)nomega * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (is_device_ptr(Sw)) {
        std::vector<float> cur(nomega);
        CK(cudaMemcpy(cur.data(), Sw, (size_t)nomega * 4, cudaMemcpyDeviceToHost));
        for (int i = 0; i < nomega; i++) cur[i] += (float)h[i];
        CK(cudaMemcpy(Sw, cur.data(), (size_t)nomega * 4, cudaMemcpyHostToDevice));
    } else {
        for (int i = 0; i < nomega; i++) Sw[i] += (float)h[i];
    }
    return CIR_OK;
}

// Frequency axis and intensity rows of the three lineshape files (calcIR.cu:890-919);
// y = C2R transform (length n) of one damped TCF.
static int lineshape_rows(const cir_params *p, const double *y, float *omega, float *inten) {
    const int n = p->ntcfpoints + p->nzeros;
    const float factor = (float)(2 * CIR_PI * CIR_HBAR / (p->dt * (float)n));
    const float norm = factor * (float)n;
    int cnt = 0;
    for (int i = n / 2; i < n; i++) {
        const float freq = -1 * (i - p->ntcfpoints - p->nzeros) * factor + p->avef;
        if (freq <= (float)p->omegaStop) {
            if (omega) omega[cnt] = freq;
            if (inten) inten[cnt] = (float)y[i] / norm;
            cnt++;
        }
    }
    for (int i = 0; i < p->ntcfpoints + p->nzeros / 2; i++) {
        const float freq = -1 * i * factor + p->avef;
        if (freq >= (float)p->omegaStart) {
            if (omega) omega[cnt] = freq;
            if (inten) inten[cnt] = (float)y[i] / norm;
            cnt++;
        }
    }
    return cnt;
}

static int c2r_dev(cir_ctx *c, const double *tcf_host, std::vector<double> &y) {
    const int n = c->p.ntcfpoints + c->p.nzeros;
    const int nx = c->p.ntcfpoints;
    CK(c->buf[B_FFT0].ensure((size_t)n * 16));
    CK(c->buf[B_FFT1].ensure((size_t)n * 16));
    CK(c->buf[B_FFTY].ensure((size_t)n * 8));
    CK(c->buf[B_FFTX].ensure((size_t)nx * 16));
    CK(cudaMemcpyAsync(c->buf[B_FFTX].p, tcf_host, (size_t)nx * 16, cudaMemcpyHostToDevice, c->stream));
    int launches = 0;
    CK(cir_launch_c2r(c->buf[B_FFTX].as<double>(), nx, n, c->buf[B_FFT0].as<double>(), c->buf[B_FFT1].as<double>(),
                      c->buf[B_FFTY].as<double>(), c->stream, &launches));
    count_launch(c, launches);
    y.resize(n);
    CK(cudaMemcpyAsync(y.data(), c->buf[B_FFTY].p, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CIR_OK;
}

extern "C" int cir_lineshape(cir_ctx *c, const double *tcf, float *omega, float *intensity, int *nls) {
    if (!c || !tcf) return cir_fail(CIR_ERR_ARG, "cir_lineshape: bad argument");
    std::vector<double> y;
    int rc = c2r_dev(c, tcf, y);
    if (rc) return rc;
    const int cnt = lineshape_rows(&c->p, y.data(), omega, intensity);
    if (nls) *nls = cnt;
    return CIR_OK;
}

namespace {
__global__ void k_gather_frames(const float *xyz, const float *box, const int *fidx, int natoms, int s_count,
                                int kn, int K, int k0, float *oxyz, float *obox) {
    const int b = blockIdx.y;                     // b = s*kn + (k - k0)
    const int s = b / kn, k = k0 + b % kn;
    const int f = fidx[s * K + k];
    const float *src = xyz + (size_t)f * natoms * 3;
    float *dst = oxyz + (size_t)b * natoms * 3;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < natoms * 3; i += gridDim.x * blockDim.x) dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x < 3) obox[3 * b + threadIdx.x] = box[3 * f + threadIdx.x];
}
__global__ void k_copy_m0(const float *m, long long sm_origin, int rows_ld, float *m0) {
    const int s = blockIdx.y;
    const float *src = m + (size_t)s * sm_origin;
    float *dst = m0 + (size_t)s * 9 * rows_ld;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 9 * rows_ld; i += gridDim.x * blockDim.x) dst[i] = src[i];
}
}  // namespace

// Launch key of a captured step loop: every shape and pointer its launches depend on.
static std::vector<long long> step_key(const Group &g, int St, int K, int k0, int kc, int precision, const void *A,
                                       const void *W, const void *M, const void *F, const void *G, const void *M0,
                                       const void *tcf, int tile1, int tile2, const void *VS, const void *FS) {
    return {g.n, g.ld, St, K, k0, kc, precision, (long long)(uintptr_t)A, (long long)(uintptr_t)W,
            (long long)(uintptr_t)M, (long long)(uintptr_t)F, (long long)(uintptr_t)G, (long long)(uintptr_t)M0,
            (long long)(uintptr_t)tcf, tile1, tile2, (long long)(uintptr_t)VS, (long long)(uintptr_t)FS};
}

static int psi_propagate(cir_ctx *c, int S, int n, int ld, const float *V, long long sV, const float *w, long long sw,
                         float dt, float *x, float *tmp, int &launches);

// CIR_EIG_SPLIT=0: the eigensolver batch of a chunk in one stream, not two (for comparison)
static bool eig_split_enabled() {
    static const bool on = [] {
        const char *v = getenv("CIR_EIG_SPLIT");
        return !(v && v[0] == '0');
    }();
    return on;
}

// Thread blocks of the tridiagonalisation of order n resident at a time (one per matrix).
static int tridiag_wave(cir_ctx *c, int n) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 1;
    auto it = c->tq_blocks.find(n);
    const int blocks = it != c->tq_blocks.end() && it->second > 0 ? it->second : cir_tridiag_blocks(n);
    return std::max(1, sms * blocks);
}

static int plan_chunk(int K, int St, int kn_max, int wave) { return cir_plan_chunk(K, St, kn_max, wave); }

// One group's job: ntraj trajectories of one size, nsamples origins each, batched through
// every launch.  dxyz / dbox hold all the group's frames on the device; fidx[(t*S + s)*K + k]
// is the frame of step k of origin s of trajectory t; res[t] receives trajectory t's results.
// The job runs in phases -- setup, then per chunk of kn steps the preparation (gather, build,
// eigensolve, step-0 work) and the step loop, then finish -- so that several groups can run
// their step loops in joint launches (run_groups_joint).  buf is the job's own device buffers
// (the context's for a single group).
struct GroupJob {
    cir_ctx *c;
    DevBuf *buf;
    DevBuf *scr;   // the preparation's scratch (frames, tables, eigensolver work areas): buf, or
                   // buffers that the groups of a joint run share, since their preparations
                   // run one after another on the stream
    Group g;
    const float *dxyz, *dbox;
    const std::vector<int> &fidx;
    cir_result *res;
    const cir_params &p;
    cudaEvent_t *ev;
    int S = 0, K = 0, n = 0, ld = 0, T = 0, St = 0, nomega = 0, kn = 0, nb = 0, ldh = 0;
    long long steps = 0, mstride = 0, vs_el = 0, fs_el = 0;
    bool vectors = false, split = false;
    float *A = nullptr, *W = nullptr, *M = nullptr, *F = nullptr, *G = nullptr, *M0 = nullptr;
    __nv_bfloat16 *vs = nullptr, *fs = nullptr;
    SplitMat Vc{}, Vr{}, Ft{}, Gt{};
    double *tcf = nullptr;
    int tile1 = 0, tile2 = 0, stile1 = 0, stile2 = 0;
    int launches = 0;
    int k0 = 0, kc = 0, nmat = 0, base0 = 0, dlt = 0;   // the chunk being run

    GroupJob(cir_ctx *c_, DevBuf *buf_, const Group &g_, const float *dxyz_, const float *dbox_,
             const std::vector<int> &fidx_, cir_result *res_)
        : c(c_), buf(buf_), scr(buf_), g(g_), dxyz(dxyz_), dbox(dbox_), fidx(fidx_), res(res_), p(c_->p),
          ev(c_->ev) {}

    // bytes of device memory one origin-step of a chunk holds from its preparation to the end
    // of its step loop (V, the eigenvalues, dipoles and polarisabilities, the status) ...
    static size_t resident_step_bytes(const cir_params &p, const Group &g) {
        return (size_t)g.n * g.ld * 4 + (size_t)(9 + 1) * g.ld * 4 + cir_eigh_de_bytes(g.ld) + 4;
    }
    // ... and during its preparation only (frames, tables, the eigensolver's work areas)
    static size_t scratch_step_bytes(const cir_params &p, const Group &g) {
        return (size_t)(p.refine_eigen > 0 ? 2 : 1) * g.n * g.ld * 4 + cir_dc_bytes(g.n, g.ld) +
               (size_t)CT_NROW * g.ld * 4 + (size_t)g.natoms * 12 + 60;
    }
    static size_t per_step_bytes(const cir_params &p, const Group &g) {
        return resident_step_bytes(p, g) + scratch_step_bytes(p, g);
    }

    // buffers, zeroed sums, tuned products; kn_set > 0 fixes the chunk length
    int setup(int kn_set) {
        S = p.nsamples; K = p.ntcfpoints; n = g.n; ld = g.ld; T = g.ntraj;
        St = S * T;                                    // origins of the group
        nomega = cir_nomega(&p);
        steps = (long long)St * K;

        // chunk: kn consecutive steps of all St origins per batch
        const size_t per_step = per_step_bytes(p, g);
        size_t budget = (size_t)64 << 30;
        size_t freeb = 0, totalb = 0;
        if (cudaMemGetInfo(&freeb, &totalb) == cudaSuccess) budget = std::min(budget, freeb / 2);
        kn = (int)std::min<size_t>((size_t)K, std::max<size_t>(1, budget / (per_step * St)));
        kn = std::max(1, std::min(kn, 65535 / std::max(1, St)));   // matrices of a chunk index a grid dimension
        kn = plan_chunk(K, St, kn, tridiag_wave(c, n));
        if (p.batch_frames > 0) kn = std::max(1, p.batch_frames / St);
        if (kn_set > 0) kn = kn_set;   // chosen by the caller for several groups together
        kn = std::min(kn, K);
        kn = std::max(1, std::min(kn, 65535 / std::max(1, St)));
        if (St > 65535) return cir_fail(CIR_ERR_ARG, "%d time origins in one group (at most 65535)", St);

        CK(buf[B_FIDX].ensure((size_t)steps * 4));
        CK(cudaMemcpyAsync(buf[B_FIDX].p, fidx.data(), (size_t)steps * 4, cudaMemcpyHostToDevice, c->stream));
        nb = St * kn;
        mstride = (long long)n * ld;
        CK(scr[B_CXYZ].ensure((size_t)nb * g.natoms * 12));
        CK(scr[B_CBOX].ensure((size_t)nb * 12));
        CK(scr[B_CT].ensure((size_t)nb * CT_NROW * ld * 4));
        CK(buf[B_A].ensure((size_t)nb * mstride * 4));
        CK(scr[B_Z].ensure((size_t)nb * mstride * 4));
        CK(scr[B_DC].ensure((size_t)nb * cir_dc_bytes(n, ld)));
        CK(buf[B_DE].ensure((size_t)nb * cir_eigh_de_bytes(ld)));   // d, e, tau: from the tridiagonalisation,
                                                                   // which may run for several groups at once
        CK(buf[B_W].ensure((size_t)nb * ld * 4));
        CK(buf[B_M].ensure((size_t)nb * 9 * ld * 4));
        CK(buf[B_STATUS].ensure((size_t)nb * 4));
        // the split-BF16 form propagates pre-split operands (k_tc_split.cu): per origin the
        // step's V as Vc and Vr and the transposed F and G, each a hi/lo pair of order ldh
        vectors = p.propagate_vectors != 0;   // psi = F m(0) instead of F
        split = !vectors && p.precision == CIR_PREC_BF16X3;
        ldh = (int)cir_split_ld(n);
        vs_el = (long long)n * ldh;
        fs_el = (long long)2 * n * ldh;   // elements per origin
        if (vectors) {
            CK(buf[B_PSI].ensure((size_t)St * n * CIR_PSI_LD * 4));
            CK(buf[B_LAM].ensure((size_t)St * n * CIR_PSI_LD * 4));
        } else if (split) {
            CK(buf[B_VS].ensure((size_t)4 * St * vs_el * 2));
            CK(buf[B_FS].ensure((size_t)4 * St * fs_el * 2));
        } else {
            CK(buf[B_F].ensure((size_t)St * n * 2 * ld * 4));
            CK(buf[B_G].ensure((size_t)St * n * 2 * ld * 4));
        }
        CK(buf[B_M0].ensure((size_t)St * 9 * ld * 4));
        CK(buf[B_TCF].ensure((size_t)steps * 6 * 8));
        CK(buf[B_HCNT].ensure((size_t)T * nomega * 8));
        CK(buf[B_HIPR].ensure((size_t)T * nomega * 8));
        CK(buf[B_HMIPR].ensure((size_t)T * nomega * 8));
        CK(buf[B_OOR].ensure((size_t)T * 8));
        CK(buf[B_SWEEPS].ensure(8));
        CK(buf[B_SW].ensure((size_t)T * nomega * 8));
        CK(buf[B_MU2].ensure((size_t)ld * 4));
        CK(cudaMemsetAsync(buf[B_TCF].p, 0, (size_t)steps * 48, c->stream));
        CK(cudaMemsetAsync(buf[B_HCNT].p, 0, (size_t)T * nomega * 8, c->stream));
        CK(cudaMemsetAsync(buf[B_HIPR].p, 0, (size_t)T * nomega * 8, c->stream));
        CK(cudaMemsetAsync(buf[B_HMIPR].p, 0, (size_t)T * nomega * 8, c->stream));
        CK(cudaMemsetAsync(buf[B_OOR].p, 0, (size_t)T * 8, c->stream));
        CK(cudaMemsetAsync(buf[B_SWEEPS].p, 0, 8, c->stream));
        CK(cudaMemsetAsync(buf[B_SW].p, 0, (size_t)T * nomega * 8, c->stream));
        CK(cudaMemsetAsync(buf[B_STATUS].p, 0, (size_t)nb * 4, c->stream));

        A = buf[B_A].as<float>();
        W = buf[B_W].as<float>();
        M = buf[B_M].as<float>();
        F = buf[B_F].as<float>();
        G = buf[B_G].as<float>();
        M0 = buf[B_M0].as<float>();
        vs = split ? buf[B_VS].as<__nv_bfloat16>() : nullptr;
        fs = split ? buf[B_FS].as<__nv_bfloat16>() : nullptr;
        Vc = SplitMat{vs, vs + St * vs_el};
        Vr = SplitMat{vs + 2 * St * vs_el, vs + 3 * St * vs_el};
        Ft = SplitMat{fs, fs + St * fs_el};
        Gt = SplitMat{fs + 2 * St * fs_el, fs + 3 * St * fs_el};
        tcf = buf[B_TCF].as<double>();
        launches = 0;
        int rc;

        // the propagation products of this group, tuned before anything is timed or captured
        GemmArgs g1{}, g2{};
        g1.M = n; g1.N = 2 * n; g1.K = n; g1.lda = ld; g1.ldb = g1.ldc = 2 * ld; g1.a_colmajor = false; g1.epilogue = 1;
        g2 = g1; g2.a_colmajor = true; g2.epilogue = 0;
        if (p.precision == CIR_PREC_FP32) {
            if ((rc = autotune_gemm(c, g1, St))) return rc;
            if ((rc = autotune_gemm(c, g2, St))) return rc;
        }
        tile1 = tuned_tile(c, g1, St);
        tile2 = tuned_tile(c, g2, St);
        // the split-BF16 products' tile widths (the shapes and strides of the step loop's two
        // products; the autotuner runs them on scratch operands)
        stile1 = stile2 = 0;
        if (split) {
            SplitGemmArgs r1{};
            r1.lda = r1.ldb = r1.ldc = ldh; r1.sA = vs_el; r1.sB = r1.sC = fs_el;
            r1.M = n; r1.N = 2 * n; r1.K = n; r1.epilogue = 1; r1.wstride = std::min(kn, K) * ld;
            r1.dt_over_hbar = (float)(p.dt / CIR_HBAR);
            r1.err = c->buf[B_ERR].as<int>();
            SplitGemmArgs r2 = r1;
            r2.epilogue = 0;
            r2.tcf_sm0 = 9LL * ld; r2.tcf_smt = (long long)std::min(kn, K) * 9 * ld; r2.tcf_ldv = ld;
            r2.tcf_sout = (long long)K * 6;
            r2.tcf_out = tcf;   // marks the fused form; the autotuner substitutes scratch
            if ((rc = autotune_split(c, r1, St))) return rc;
            if ((rc = autotune_split(c, r2, St))) return rc;
            stile1 = tuned_split(c, r1, St);
            stile2 = tuned_split(c, r2, St);
        }
        return CIR_OK;
    }

    // the chunk of steps k0_ .. k0_ + kc_ - 1: frames gathered, Hamiltonians built and
    // diagonalised, the distributions binned; at step 0 the spectral density and F = I.
    // Records ev[1] (start), ev[2] (built), ev[5] (tridiagonalised), ev[3] (done); with
    // account, waits for ev[3] and adds the build and eigensolver times to the stats.
    int prepare(int k0_, int kc_, bool account) {
        int rc;
        if ((rc = prepare_build(k0_, kc_, true))) return rc;
        if ((rc = prepare_eig(false, true))) return rc;
        if (account) {   // this group's build and eigensolve time, read now (the events are reused)
            CK(cudaEventSynchronize(ev[3]));
            float x;
            cudaEventElapsedTime(&x, ev[1], ev[2]);
            c->stats.ms_build += x;
            cudaEventElapsedTime(&x, ev[2], ev[3]);
            c->stats.ms_eig += x;
            x = tridiag_ms();
            c->stats.ms_tridiag += x;
            if (p.verbose > 1) printf("  order %d, steps %d..%d: tridiagonalisation %.1f ms\n", n, k0, k0 + kc - 1, x);
        }
        return CIR_OK;
    }

    EighArgs eg{};   // the chunk's eigensolver arguments (prepare_build)

    bool split_done = false;   // the last prepare_eig ran two parts (split_eig)

    // ms from the end of the build (ev[2]) to the end of the tridiagonalisation: of the later
    // part when the batch ran in two (the events are complete once ev[3] is)
    float tridiag_ms() const {
        float x = 0.f;
        cudaEventElapsedTime(&x, ev[2], ev[5]);
        if (split_done) {
            float y = 0.f, z = 0.f;
            cudaEventElapsedTime(&y, ev[2], c->xev[1]);
            if (p.verbose > 1) {
                cudaEventElapsedTime(&z, ev[2], ev[3]);
                printf("  two parts: tridiagonalisations end at %.1f and %.1f ms, eigensolver at %.1f ms\n", x, y, z);
            }
            x = std::max(x, y);
        }
        return x;
    }

    // eg over matrices [0, hA) on the library stream and [hA, nmat) on c->aux, joined before
    // the library stream goes on; the two tridiagonalisations end at ev[5] and c->xev[1]
    int split_eig(int hA) {
        if (!c->aux) {
            int lo = 0, hi = 0;
            CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            CK(cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, lo));
            for (auto &x : c->xev) CK(cudaEventCreate(&x));
        }
        const int hB = nmat - hA;
        EighArgs a = eg, b = eg;
        a.tq_done = ev[5];
        b.tq_done = c->xev[1];
        b.A = eg.A + (size_t)hA * mstride;
        b.W = eg.W + (size_t)hA * eg.wstride;
        b.Z = eg.Z + (size_t)hA * mstride;
        b.DE = eg.DE + (size_t)hA * 3 * ld;
        b.DC = eg.DC + (size_t)3 * hA * mstride;   // [3][hB] after the first part's [3][hA]
        b.status = eg.status + hA;
        if (eg.hist_weight) b.hist_weight = eg.hist_weight + hA;
        if (eg.hist_group) b.hist_group = 0;
        if (eg.hist_group) a.hist_group = 0;
        CK(cudaEventRecord(c->xev[0], c->stream));
        CK(cudaStreamWaitEvent(c->aux, c->xev[0], 0));
        CK(cir_launch_eigh(a, hA, c->stream, &launches));
        CK(cir_launch_eigh(b, hB, c->aux, &launches));
        CK(cudaEventRecord(c->xev[2], c->aux));
        CK(cudaStreamWaitEvent(c->stream, c->xev[2], 0));
        split_done = true;
        return CIR_OK;
    }

    // gather and build the chunk's Hamiltonians and set up eg; events: record ev[1] and ev[2]
    int prepare_build(int k0_, int kc_, bool events) {
        k0 = k0_;
        kc = kc_;
        int rc;
        const int nbc = St * kc;
        // Matrix of origin s at step k0 + kk: base0 + kk + s * dlt.  Without sharing every
        // origin has its own kc consecutive matrices (base0 = 0, dlt = kc).  With share_frames,
        // when the chunk's frames lie on that pattern over their sorted distinct list (origins
        // evenly spaced in one trajectory, as the reference places them), each distinct frame
        // is built and diagonalised once and counts in the distributions as often as it is used.
        nmat = nbc;
        base0 = 0;
        dlt = kc;
        int *ufr = nullptr;
        if (p.share_frames && T == 1 && St > 1) {
            std::vector<int> uf;
            uf.reserve(nbc);
            for (int s2 = 0; s2 < St; s2++)
                for (int kk = 0; kk < kc; kk++) uf.push_back(fidx[(size_t)s2 * K + k0 + kk]);
            std::sort(uf.begin(), uf.end());
            uf.erase(std::unique(uf.begin(), uf.end()), uf.end());
            auto pos = [&](int f) { return (int)(std::lower_bound(uf.begin(), uf.end(), f) - uf.begin()); };
            const int b0 = pos(fidx[(size_t)k0]), d = pos(fidx[(size_t)K + k0]) - b0;
            bool ok = (int)uf.size() < nbc && d > 0;
            for (int s2 = 0; ok && s2 < St; s2++)
                for (int kk = 0; ok && kk < kc; kk++) ok = pos(fidx[(size_t)s2 * K + k0 + kk]) == b0 + kk + s2 * d;
            if (ok) {
                nmat = (int)uf.size();
                base0 = b0;
                dlt = d;
                std::vector<int> wgt(nmat, 0);
                for (int s2 = 0; s2 < St; s2++)
                    for (int kk = 0; kk < kc; kk++) wgt[b0 + kk + s2 * d]++;
                CK(buf[B_UFR].ensure((size_t)nmat * 8));
                ufr = buf[B_UFR].as<int>();
                CK(cudaMemcpyAsync(ufr, uf.data(), (size_t)nmat * 4, cudaMemcpyHostToDevice, c->stream));
                CK(cudaMemcpyAsync(ufr + nmat, wgt.data(), (size_t)nmat * 4, cudaMemcpyHostToDevice, c->stream));
            }
        }
        if (events) CK(cudaEventRecord(ev[1], c->stream));
        if (ufr)
            k_gather_frames<<<dim3(8, nmat), 256, 0, c->stream>>>(dxyz, dbox, ufr, g.natoms, 1, nmat, nmat, 0,
                                                                  scr[B_CXYZ].as<float>(), scr[B_CBOX].as<float>());
        else
            k_gather_frames<<<dim3(8, nbc), 256, 0, c->stream>>>(dxyz, dbox, buf[B_FIDX].as<int>(), g.natoms, St, kc,
                                                                 K, k0, scr[B_CXYZ].as<float>(), scr[B_CBOX].as<float>());
        CK(cudaGetLastError());
        launches++;
        BuildArgs a = build_args(c, g);
        a.xyz = scr[B_CXYZ].as<float>();
        a.box = scr[B_CBOX].as<float>();
        a.ct = scr[B_CT].as<float>();
        a.H = A;
        a.ldh = ld;
        a.dip = M;                    // frame b: M + b*9*ld, rows 0..2 dipole, 3..8 polarisability
        a.pol = M + 3 * ld;
        a.ldv = ld;
        a.dip_fstride = 9LL * ld;
        a.pol_fstride = 9LL * ld;
        CK(cir_launch_build(a, nmat, c->stream, &launches));
        if (events) CK(cudaEventRecord(ev[2], c->stream));
        EighArgs &e = eg;
        memset(&e, 0, sizeof e);
        e.A = A;
        e.W = W;
        e.Z = scr[B_Z].as<float>();
        e.DC = scr[B_DC].as<float>();
        e.DE = buf[B_DE].as<float>();
        e.mstride = mstride;
        e.wstride = ld;
        e.n = n;
        e.ld = ld;
        e.status = buf[B_STATUS].as<int>();
        e.sweeps = buf[B_SWEEPS].as<unsigned long long>();
        e.hist_count = buf[B_HCNT].as<unsigned long long>();
        e.hist_ipr = buf[B_HIPR].as<double>();
        e.hist_mipr = buf[B_HMIPR].as<double>();
        e.out_of_range = buf[B_OOR].as<unsigned long long>();
        e.hist_group = ufr ? 0 : S * kc;   // the chunk's matrices of one trajectory share its histograms
        e.hist_weight = ufr ? ufr + nmat : nullptr;
        e.nomega = nomega;
        e.omegaStep = p.omegaStep;
        e.nchrom_mol = p.nchrom_mol;
        // eigenvectors need more than TF32's 10-bit mantissa: both mixed forms run the
        // eigensolver's tensor-core products as 3-pass split BF16
        e.precision = p.precision == CIR_PREC_FP32 ? CIR_PREC_FP32 : CIR_PREC_BF16X3;
        e.err = c->buf[B_ERR].as<int>();
        e.test_stall = c->p.test_stall_gemm;
        e.test_sweep_cap = c->p.test_sweep_cap;
        e.tq_done = ev[5];
        e.avef = p.avef;
        e.omegaStart = p.omegaStart;
        if (eigh_profiling()) {
            CK(c->buf[B_PROF].ensure((size_t)nmat * CIR_EIG_PROF_SLOTS * 8));
            CK(cudaMemsetAsync(c->buf[B_PROF].p, 0, (size_t)nmat * CIR_EIG_PROF_SLOTS * 8, c->stream));
            e.phase_ns = c->buf[B_PROF].as<unsigned long long>();
        }
        if (k0 == 0 && (rc = autotune_tridiag(c, e, nmat))) return rc;
        if (c->tq_blocks.count(n)) e.tq_blocks = c->tq_blocks[n];
        if ((rc = setup_refine(c, e, nmat))) return rc;
        return CIR_OK;
    }

    // the eigensolver on eg (skip_tq: its tridiagonalisation has run already) and the step-0
    // work; records ev[3] after the eigensolver
    int prepare_eig(bool skip_tq, bool may_split = false) {
        EighArgs &e = eg;
        e.skip_tridiag = skip_tq ? 1 : 0;
        split_done = false;
        int hA = 0;   // the first part: whole waves of the tridiagonalisation, all but the last one
        if (may_split && !skip_tq && eig_split_enabled() && !e.Href && !e.phase_ns &&
            (e.hist_group == 0 || e.hist_group >= nmat)) {
            hA = cir_split_first_part(nmat, tridiag_wave(c, n));
        }
        if (hA > 0 && hA < nmat) {
            // the batch in two parts on two streams: the first (whole waves) on the library
            // stream, the rest on a second one, so that the first part's divide and conquer
            // and back-transform can start while the rest is still being tridiagonalised
            int rc;
            if ((rc = split_eig(hA))) return rc;
        } else {
            CK(cir_launch_eigh(e, nmat, c->stream, &launches));
        }
        c->stats.eig_matrices += nmat;
        if (e.phase_ns) eigh_profile_report(e.phase_ns, nmat, c->stream);
        CK(cudaEventRecord(ev[3], c->stream));
        if (k0 == 0) {
            // spectral density at step 0 of every origin (calcIR.cu:456-482), per trajectory
            for (int s = 0; s < St; s++) {
                const size_t b = (size_t)base0 + (size_t)s * dlt;
                CK(cir_launch_spectral(A + b * mstride, ld, W + b * ld, M + b * 9 * ld, ld, n, buf[B_MU2].as<float>(),
                                       buf[B_SW].as<double>() + (size_t)(s / S) * nomega, nomega, p.omegaStart,
                                       p.omegaStep, p.t1, p.avef, c->stream, &launches));
            }
            // F = I and the t = 0 vectors (calcIR.cu:577-594)
            if (vectors) {
                CK(cir_adj_psi_init(M + (size_t)base0 * 9 * ld, (long long)dlt * 9 * ld, ld, n, St,
                                    buf[B_PSI].as<float>(), c->stream));
            } else {
                if (split) CK(cir_launch_identity_t(Ft, n, ldh, fs_el, St, c->stream, &launches));
                else CK(cir_launch_identity(F, n, 2 * ld, (long long)n * 2 * ld, St, c->stream, &launches));
                k_copy_m0<<<dim3(4, St), 256, 0, c->stream>>>(M + (size_t)base0 * 9 * ld, (long long)dlt * 9 * ld, ld, M0);
                CK(cudaGetLastError());
            }
            launches++;
        }
        return CIR_OK;
    }

    // the split-BF16 products of step k (k > 0): G = V^T F with the phase, F' = V G with the
    // step's correlation terms fused
    void split_step(int k, SplitGemmArgs &s1, SplitGemmArgs &s2) const {
        const size_t mk = (size_t)base0 + (k - k0);
        s1 = SplitGemmArgs{};
        s1.Ahi = Vc.hi; s1.Alo = Vc.lo; s1.lda = ldh; s1.sA = vs_el;       // V^T
        s1.Bhi = Ft.hi; s1.Blo = Ft.lo; s1.ldb = ldh; s1.sB = fs_el;       // F
        s1.Chi = Gt.hi; s1.Clo = Gt.lo; s1.ldc = ldh; s1.sC = fs_el;       // G, transposed
        s1.M = n; s1.N = 2 * n; s1.K = n;
        s1.epilogue = 1; s1.w = W + mk * ld; s1.wstride = dlt * ld;
        s1.dt_over_hbar = (float)(p.dt / CIR_HBAR);
        s1.err = c->buf[B_ERR].as<int>();
        s1.test_stall = p.test_stall_gemm;
        s2 = s1;
        s2.Ahi = Vr.hi; s2.Alo = Vr.lo;                                    // V
        s2.Bhi = Gt.hi; s2.Blo = Gt.lo;
        s2.Chi = Ft.hi; s2.Clo = Ft.lo;                                    // F', transposed
        s2.epilogue = 0;
        // the step's correlation terms fused into F' = V G
        s2.tcf_m0 = M0; s2.tcf_sm0 = 9LL * ld;
        s2.tcf_mt = M + mk * 9 * ld; s2.tcf_smt = (long long)dlt * 9 * ld; s2.tcf_ldv = ld;
        s2.tcf_out = tcf + (size_t)k * 6; s2.tcf_sout = (long long)K * 6;
        s1.tile_n = stile1;
        s2.tile_n = stile2;
    }

    // the chunk's steps: F <- V_k exp(i L_k dt/hbar) V_k^T F for every origin
    // (calcIR.cu:596-617), then the correlation terms (calcIR.cu:628-745)
    int steps_launch(int &nl) {
        for (int k = k0; k < k0 + kc; k++) {
            const int rc = step_launch(k, nl);
            if (rc) return rc;
        }
        return CIR_OK;
    }

    // step k of the chunk, every origin of the group
    int step_launch(int k, int &nl) {
        {
            const int kk = k - k0;
            const size_t mk = (size_t)base0 + kk;      // matrix of origin 0 at this step
            if (vectors) {
                if (k > 0) {
                    const int rc2 = psi_propagate(c, St, n, ld, A + mk * mstride, (long long)dlt * mstride, W + mk * ld,
                                                  (long long)dlt * ld, p.dt, buf[B_PSI].as<float>(),
                                                  buf[B_LAM].as<float>(), nl);
                    if (rc2) return rc2;
                }
                CK(cir_adj_tcf(buf[B_PSI].as<float>(), M + mk * 9 * ld, (long long)dlt * 9 * ld, ld, n, St,
                               tcf + (size_t)k * 6, (long long)K * 6, c->stream));
                nl++;
                return CIR_OK;
            }
            if (k > 0 && split) {
                CK(cir_launch_split_v(A + mk * mstride, ld, (long long)dlt * mstride, n, Vc, Vr, ldh, vs_el,
                                      St, c->stream, &nl));
                SplitGemmArgs s1, s2;
                split_step(k, s1, s2);
                CK(cir_launch_split_gemm(s1, St, c->stream, &nl));
                CK(cir_launch_split_gemm(s2, St, c->stream, &nl));
                return CIR_OK;
            } else if (k > 0) {
                int rc2 = propagate_dev(c, St, n, A + mk * mstride, ld, (long long)dlt * mstride,
                                        W + mk * ld, dlt * ld, p.dt, F, 2 * ld, (long long)n * 2 * ld, G, nl);
                if (rc2) return rc2;
            }
            TcfArgs t;
            memset(&t, 0, sizeof t);
            t.F = F;
            t.sF = (long long)n * 2 * ld;
            t.m0 = M0;
            t.sm0 = 9LL * ld;
            t.mt = M + mk * 9 * ld;
            t.smt = (long long)dlt * 9 * ld;
            t.out = tcf + (size_t)k * 6;
            t.sout = (long long)K * 6;
            t.n = n;
            t.ldf = 2 * ld;
            t.ldv = ld;
            if (split) {
                t.Ft = Ft;
                t.sFt = fs_el;
                t.ldft = ldh;
            }
            CK(cir_launch_tcf(t, St, c->stream, &nl));
        }
        return CIR_OK;
    }

    // the key of the chunk's captured step loop
    std::vector<long long> graph_key() const {
        std::vector<long long> key = step_key(g, St, K, k0, kc, p.precision, A, W, M, F, G, M0, tcf, tile1, tile2, vs, fs);
        key.insert(key.end(), {(long long)vectors, (long long)base0, (long long)dlt, (long long)stile1, (long long)stile2,
                               (long long)(uintptr_t)buf[B_PSI].p, (long long)(uintptr_t)buf[B_LAM].p});
        return key;
    }

    // results of every trajectory, after the last chunk (ms_total: the job's device time)
    int finish(float ms_total) {
        int rc;
        count_launch(c, launches);
        c->stats.frame_steps += steps;

        // results: correlation sums, histograms, spectral density of every trajectory
        std::vector<double> htcf((size_t)steps * 6), hipr((size_t)T * nomega), hmipr((size_t)T * nomega), hsw((size_t)T * nomega);
        std::vector<unsigned long long> hcnt((size_t)T * nomega), oor(T);
        std::vector<int> hst(nb);
        unsigned long long sweeps = 0;
        CK(cudaMemcpyAsync(htcf.data(), tcf, (size_t)steps * 48, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(hcnt.data(), buf[B_HCNT].p, (size_t)T * nomega * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(hipr.data(), buf[B_HIPR].p, (size_t)T * nomega * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(hmipr.data(), buf[B_HMIPR].p, (size_t)T * nomega * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(hsw.data(), buf[B_SW].p, (size_t)T * nomega * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(hst.data(), buf[B_STATUS].p, (size_t)nb * 4, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(oor.data(), buf[B_OOR].p, (size_t)T * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(&sweeps, buf[B_SWEEPS].p, 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->stats.eig_sweeps += (long long)sweeps;
        for (int i = 0; i < nb; i++)
            if (hst[i]) return cir_fail(CIR_ERR_NOCONVERGE, "eigensolver sweep cap reached");
        if (p.precision != CIR_PREC_FP32 && (rc = check_kernel_flag(c))) return rc;

        for (int tr = 0; tr < T; tr++) {
            cir_result *r = res + tr;
            const double *sw_t = hsw.data() + (size_t)tr * nomega, *ipr_t = hipr.data() + (size_t)tr * nomega,
                         *mipr_t = hmipr.data() + (size_t)tr * nomega;
            const unsigned long long *cnt_t = hcnt.data() + (size_t)tr * nomega;
            // sum over origins, T1 damping and 1/nsamples (calcIR.cu:777-782, 798-802, 815-819)
            std::vector<double> damped[3];
            for (int q = 0; q < 3; q++) damped[q].assign((size_t)2 * K, 0.0);
            for (int k = 0; k < K; k++) {
                CompSum sum[6];
                for (int s = tr * S; s < (tr + 1) * S; s++)
                    for (int q = 0; q < 6; q++) sum[q].add(htcf[((size_t)s * K + k) * 6 + q]);
                const double dcy = exp(-1.0 * k * p.dt / (2.0 * p.t1)) / (1. * S);
                for (int q = 0; q < 3; q++) {
                    damped[q][2 * k] = sum[2 * q].value() * dcy;
                    damped[q][2 * k + 1] = sum[2 * q + 1].value() * dcy;
                }
            }
            double *outs[3] = {r->tcf_ir, r->tcf_vv, r->tcf_vh};
            for (int q = 0; q < 3; q++)
                if (outs[q]) memcpy(outs[q], damped[q].data(), (size_t)2 * K * 8);
            // spectral density and frequency distributions (calcIR.cu:831-839)
            const float norm = (float)(n * S * K);
            for (int i = 0; i < nomega; i++) {
                if (r->omega) r->omega[i] = (float)(p.omegaStart + p.omegaStep * i);
                if (r->sw) r->sw[i] = (float)(sw_t[i] / S);
                const float pw = (float)((double)cnt_t[i] / p.omegaStep) / norm;
                if (r->pw) r->pw[i] = pw;
                if (r->rw) r->rw[i] = ((float)(ipr_t[i] / p.omegaStep) / norm) / pw;
                if (r->rmw) r->rmw[i] = ((float)(mipr_t[i] / p.omegaStep) / norm) / pw;
            }
            // lineshapes (calcIR.cu:786-827, 890-919)
            float *lsv[3] = {r->ls_ir, r->ls_vv, r->ls_vh};
            int nls = 0;
            for (int q = 0; q < 3; q++) {
                std::vector<double> y;
                int rc3 = c2r_dev(c, damped[q].data(), y);
                if (rc3) return rc3;
                nls = lineshape_rows(&p, y.data(), q == 0 ? r->ls_omega : nullptr, lsv[q]);
            }
            r->nls = nls;
            r->bins_out_of_range = (long long)oor[tr];
            r->frame_steps_per_s = ms_total > 0 ? steps / (ms_total * 1e-3) : 0.0;
        }
        return CIR_OK;
    }
};

// The step loop of a chunk: replayed from a captured CUDA graph (cached by key) when the
// context uses graphs, else launched directly.
static int step_loop(cir_ctx *c, const std::vector<long long> &key, const std::function<int(int &)> &launch,
                     int &launches) {
    if (!c->p.cuda_graphs) {
        int nl = 0;
        const int rc = launch(nl);
        launches += nl;
        return rc;
    }
    GraphEntry *ge = nullptr;
    for (auto &x : c->graphs)
        if (x.key == key) ge = &x;
    if (!ge) {
        int nl = 0;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int rc2 = launch(nl);
        cudaGraph_t gr = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(c->stream, &gr);
        if (rc2) {
            if (gr) cudaGraphDestroy(gr);
            return rc2;
        }
        if (ce != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "capturing the step loop: %s", cudaGetErrorString(ce));
        GraphEntry ne;
        ne.key = key;
        ne.launches = nl;
        const cudaError_t ie = cudaGraphInstantiate(&ne.exec, gr, 0);
        cudaGraphDestroy(gr);
        if (ie != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "instantiating the step loop: %s", cudaGetErrorString(ie));
        if (c->graphs.size() >= 32) {
            cudaGraphExecDestroy(c->graphs.front().exec);
            c->graphs.erase(c->graphs.begin());
        }
        c->graphs.push_back(ne);
        ge = &c->graphs.back();
    }
    CK(cudaGraphLaunch(ge->exec, c->stream));
    launches += ge->launches;
    return CIR_OK;
}

// The frame-steps of one group (see GroupJob), with the context's buffers.
static int run_group(cir_ctx *c, const Group &g, const float *dxyz, const float *dbox, const std::vector<int> &fidx,
                     cir_result *res, double *ms_run) {
    GroupJob j(c, c->buf, g, dxyz, dbox, fidx, res);
    int rc;
    if ((rc = j.setup(0))) return rc;
    if (c->p.verbose > 1)
        printf("group of %d chromophores: %d origins, chunks of %d steps\n", j.n, j.St, j.kn);
    cudaEvent_t *ev = c->ev;
    CK(cudaEventRecord(ev[0], c->stream));
    for (int k0 = 0; k0 < j.K; k0 += j.kn) {
        if ((rc = j.prepare(k0, std::min(j.kn, j.K - k0), false))) return rc;
        if ((rc = step_loop(c, j.graph_key(), [&](int &nl) { return j.steps_launch(nl); }, j.launches))) return rc;
        CK(cudaEventRecord(ev[4], c->stream));
        CK(cudaEventSynchronize(ev[4]));
        float x;
        cudaEventElapsedTime(&x, ev[1], ev[2]);
        c->stats.ms_build += x;
        cudaEventElapsedTime(&x, ev[2], ev[3]);
        c->stats.ms_eig += x;
        x = j.tridiag_ms();
        c->stats.ms_tridiag += x;
        if (c->p.verbose > 1) printf("  order %d, steps %d..%d: tridiagonalisation %.1f ms\n", j.n, k0, k0 + j.kc - 1, x);
        cudaEventElapsedTime(&x, ev[3], ev[4]);
        c->stats.ms_prop += x;
    }
    CK(cudaEventRecord(ev[7], c->stream));
    CK(cudaEventSynchronize(ev[7]));
    float ms_total = 0;
    cudaEventElapsedTime(&ms_total, ev[0], ev[7]);
    if (ms_run) *ms_run = ms_total;
    return j.finish(ms_total);
}

// Whether cir_run_multi runs the step loops of its size groups jointly (CIR_JOINT=0: one
// group after another, for comparison).
static bool joint_enabled() {
    static const bool on = [] {
        const char *v = getenv("CIR_JOINT");
        return !(v && v[0] == '0');
    }();
    return on;
}

// CIR_JOINT_TQ=0: in joint runs every group tridiagonalises its own chunks (for comparison)
static bool joint_tq_enabled() {
    static const bool on = [] {
        const char *v = getenv("CIR_JOINT_TQ");
        return !(v && v[0] == '0');
    }();
    return on;
}

// The preparations of the groups whose chunks start at step k0.  When two or more of them
// have orders 257-1024 (the blocked tridiagonalisation), their Hamiltonians are built one
// group after another and tridiagonalised in one launch (cir_launch_tridiag_multi: the
// longest matrices first, the shorter ones filling the last wave, each group's panel W in
// one shared area), then each group's eigensolver goes on from its d, e and reflectors;
// otherwise group by group.  The build time counted includes the autotuner's trials of the
// first chunk.
static int prepare_segment(cir_ctx *c, std::vector<std::unique_ptr<GroupJob>> &jobs, const std::vector<int> &prep,
                           int k0) {
    const int K = c->p.ntcfpoints;
    int rc;
    std::vector<int> jt;
    // (not with the eigenpair refinement, whose copy of the input matrices is one shared area)
    if (joint_tq_enabled() && !eigh_profiling() && c->p.refine_eigen <= 0)
        for (int i : prep)
            if (jobs[i]->n > 256 && jobs[i]->n <= 1024) jt.push_back(i);
    if (jt.size() < 2) {
        for (int i : prep) {
            GroupJob &j = *jobs[i];
            if ((rc = j.prepare(k0, std::min(j.kn, K - k0), true))) return rc;
        }
        return CIR_OK;
    }
    cudaEvent_t *ev = c->ev;
    CK(cudaEventRecord(ev[1], c->stream));
    for (int i : prep) {
        GroupJob &j = *jobs[i];
        if ((rc = j.prepare_build(k0, std::min(j.kn, K - k0), false))) return rc;
        j.eg.tq_done = nullptr;
    }
    CK(cudaEventRecord(ev[2], c->stream));
    size_t wf = 0;
    for (int i : jt) wf += (size_t)jobs[i]->nmat * cir_tridiag_w_floats(jobs[i]->ld);
    CK(c->buf[B_TQW].ensure(wf * 4));
    EighArgs a[CIR_TQ_MAXP];
    int nm[CIR_TQ_MAXP];
    size_t off = 0;
    for (size_t q = 0; q < jt.size(); q++) {
        GroupJob &j = *jobs[jt[q]];
        a[q] = j.eg;
        a[q].Z = c->buf[B_TQW].as<float>() + off;
        a[q].zstride = (long long)cir_tridiag_w_floats(j.ld);
        nm[q] = j.nmat;
        off += (size_t)j.nmat * a[q].zstride;
    }
    CK(cir_launch_tridiag_multi(a, nm, (int)jt.size(), c->stream, &jobs[jt[0]]->launches));
    CK(cudaEventRecord(ev[5], c->stream));
    for (int i : prep)
        if ((rc = jobs[i]->prepare_eig(std::find(jt.begin(), jt.end(), i) != jt.end(), false))) return rc;
    CK(cudaEventRecord(ev[3], c->stream));
    CK(cudaEventSynchronize(ev[3]));
    float x;
    cudaEventElapsedTime(&x, ev[1], ev[2]);
    c->stats.ms_build += x;
    cudaEventElapsedTime(&x, ev[2], ev[3]);
    c->stats.ms_eig += x;
    cudaEventElapsedTime(&x, ev[2], ev[5]);
    c->stats.ms_tridiag += x;
    if (c->p.verbose > 1) {
        printf("  steps %d..: one tridiagonalisation launch for orders", k0);
        for (int i : jt) printf(" %d (%d matrices)", jobs[i]->n, jobs[i]->nmat);
        printf(": %.1f ms\n", x);
    }
    return CIR_OK;
}

// Up to CIR_SPLIT_MAXP size groups of one cir_run_multi job in the split-BF16 form, run in
// lockstep: per chunk every group's frames are built and diagonalised with its own buffers,
// then each step of the chunk is one persistent launch of G = V^T F over the origins of all
// groups and one of F' = V G (each group's correlation terms fused into its tiles), after a
// small launch per group that splits the step's V into BF16 pairs.  Boxes of different size
// thus share every propagation launch.  Each group keeps the chunk length it would take
// alone; the steps run jointly up to the first end of a prepared chunk, where that group
// prepares its next one.
static int run_groups_joint(cir_ctx *c, std::vector<std::unique_ptr<GroupJob>> &jobs) {
    const cir_params &p = c->p;
    const int K = p.ntcfpoints, ng = (int)jobs.size();
    // chunk lengths: each group takes the chunks it would take alone (up to 64 GiB, planned
    // by plan_chunk against the tridiagonalisation's waves).  The groups' chunks are resident together, but only V, the eigenvalues and the
    // dipoles stay from a preparation to the end of its step loop: the preparations run one
    // after another and share one scratch (frames, tables, the eigensolver's work areas), so
    // a run holds the sum of the resident parts and the largest scratch; when that exceeds
    // 60% of the free memory every group's share shrinks in proportion
    size_t freeb = 0, totalb = 0;
    size_t budget = (size_t)64 << 30;
    if (cudaMemGetInfo(&freeb, &totalb) == cudaSuccess) budget = std::min(budget * ng, freeb / 10 * 6);
    std::vector<size_t> per(ng), res(ng), scr(ng);
    for (int i = 0; i < ng; i++) {
        const size_t st = (size_t)(p.nsamples * jobs[i]->g.ntraj);
        per[i] = GroupJob::per_step_bytes(p, jobs[i]->g) * st;
        res[i] = GroupJob::resident_step_bytes(p, jobs[i]->g) * st;
        scr[i] = GroupJob::scratch_step_bytes(p, jobs[i]->g) * st;
        jobs[i]->scr = c->buf;
    }
    auto balanced = [&](double cap_bytes, int i) {
        const int St = p.nsamples * jobs[i]->g.ntraj;
        if (p.batch_frames > 0) return std::max(1, std::min(K, p.batch_frames / St));
        int km = (int)std::max(1.0, std::min((double)K, cap_bytes / (double)per[i]));
        km = std::max(1, std::min(km, 65535 / std::max(1, St)));
        return plan_chunk(K, St, km, tridiag_wave(c, jobs[i]->g.n));
    };
    std::vector<int> kn(ng);
    double cap = (double)((size_t)64 << 30);
    for (int it = 0; it < 64; it++, cap *= 0.9) {
        size_t total = 0, smax = 0;
        for (int i = 0; i < ng; i++) {
            kn[i] = balanced(cap, i);
            total += (size_t)kn[i] * res[i];
            smax = std::max(smax, (size_t)kn[i] * scr[i]);
        }
        if (total + smax <= budget) break;
    }
    int rc;
    for (int i = 0; i < ng; i++) {
        if ((rc = jobs[i]->setup(kn[i]))) return rc;   // setup may shorten kn (grid limits)
        if (p.verbose)
            printf("joint group of %d chromophores: %d origins, chunks of %d steps\n", jobs[i]->n, jobs[i]->St,
                   jobs[i]->kn);
    }
    cudaEvent_t *ev = c->ev;
    int launches = 0;
    std::vector<int> next(ng, 0);   // first step not covered by each group's prepared chunk
    CK(cudaEventRecord(ev[0], c->stream));
    for (int k0 = 0; k0 < K;) {
        std::vector<int> prep;
        for (int i = 0; i < ng; i++)
            if (next[i] == k0) prep.push_back(i);
        if ((rc = prepare_segment(c, jobs, prep, k0))) return rc;
        for (int i : prep) next[i] = k0 + jobs[i]->kc;
        const int k1 = *std::min_element(next.begin(), next.end());   // steps k0 .. k1 - 1 run jointly
        CK(cudaEventRecord(ev[3], c->stream));
        std::vector<long long> key = {-1, ng, k0, k1};
        for (auto &j : jobs) {
            const std::vector<long long> kj = j->graph_key();
            key.insert(key.end(), kj.begin(), kj.end());
        }
        auto launch = [&](int &nl) -> int {
            for (int k = k0; k < k1; k++) {
                if (k == 0) {   // the step-0 correlation terms of every group (F = I)
                    for (auto &j : jobs)
                        if (int r = j->step_launch(0, nl)) return r;
                    continue;
                }
                SplitGemmArgs s1[CIR_SPLIT_MAXP], s2[CIR_SPLIT_MAXP];
                int batch[CIR_SPLIT_MAXP];
                for (int i = 0; i < ng; i++) {
                    GroupJob &j = *jobs[i];
                    const size_t mk = (size_t)j.base0 + (k - j.k0);
                    CK(cir_launch_split_v(j.A + mk * j.mstride, j.ld, (long long)j.dlt * j.mstride, j.n, j.Vc, j.Vr, j.ldh,
                                          j.vs_el, j.St, c->stream, &nl));
                    j.split_step(k, s1[i], s2[i]);
                    batch[i] = j.St;
                }
                CK(cir_launch_split_gemm_multi(s1, batch, ng, c->stream, &nl));
                CK(cir_launch_split_gemm_multi(s2, batch, ng, c->stream, &nl));
            }
            return CIR_OK;
        };
        if ((rc = step_loop(c, key, launch, launches))) return rc;
        CK(cudaEventRecord(ev[4], c->stream));
        CK(cudaEventSynchronize(ev[4]));
        float x;
        cudaEventElapsedTime(&x, ev[3], ev[4]);
        c->stats.ms_prop += x;
        k0 = k1;
    }
    CK(cudaEventRecord(ev[7], c->stream));
    CK(cudaEventSynchronize(ev[7]));
    float ms_total = 0;
    cudaEventElapsedTime(&ms_total, ev[0], ev[7]);
    count_launch(c, launches);
    for (auto &j : jobs)
        if ((rc = j->finish(ms_total))) return rc;
    return CIR_OK;
}

extern "C" int cir_run(cir_ctx *c, int nframes, const float *xyz, const float *box, const int *frame_of_step,
                       cir_result *r) {
    if (!c || !xyz || !box || !r || nframes < 1) return cir_fail(CIR_ERR_ARG, "cir_run: bad argument");
    const cir_params &p = c->p;
    const long long steps = (long long)p.nsamples * p.ntcfpoints;
    std::vector<int> fidx(steps);
    if (frame_of_step) {
        for (long long i = 0; i < steps; i++) {
            if (frame_of_step[i] < 0 || frame_of_step[i] >= nframes)
                return cir_fail(CIR_ERR_ARG, "frame_of_step[%lld] = %d outside [0, %d)", i, frame_of_step[i], nframes);
            fidx[i] = frame_of_step[i];
        }
    } else {
        if (nframes != steps) return cir_fail(CIR_ERR_ARG, "cir_run: %d frames for %lld frame-steps", nframes, steps);
        for (long long i = 0; i < steps; i++) fidx[i] = (int)i;
    }
    const size_t nx = (size_t)nframes * c->natoms * 3;
    if (!is_device_ptr(xyz) && !all_finite(xyz, nx)) return cir_fail(CIR_ERR_NONFINITE, "positions contain NaN or Inf");
    if (!is_device_ptr(box) && !all_finite(box, 3 * (size_t)nframes)) return cir_fail(CIR_ERR_NONFINITE, "box contains NaN or Inf");
    void *dxyz, *dbox;
    int rc;
    if ((rc = stage_in(c, B_XYZ, xyz, nx * 4, &dxyz, true))) return rc;
    if ((rc = stage_in(c, B_BOX, box, (size_t)nframes * 12, &dbox, true))) return rc;
    return run_group(c, ctx_group(c), static_cast<const float *>(dxyz), static_cast<const float *>(dbox), fidx, r, nullptr);
}

extern "C" int cir_run_multi(cir_ctx *c, int ntraj, const cir_traj_in *traj, cir_result *results) {
    if (!c || ntraj < 1 || !traj || !results) return cir_fail(CIR_ERR_ARG, "cir_run_multi: bad argument");
    const cir_params &p = c->p;
    const long long steps = (long long)p.nsamples * p.ntcfpoints;
    // groups of equal size, in order of size
    std::map<int, std::vector<int>> groups;
    for (int i = 0; i < ntraj; i++) {
        const cir_traj_in &t = traj[i];
        if (!t.xyz || !t.box || t.nframes < 1) return cir_fail(CIR_ERR_ARG, "cir_run_multi: trajectory %d: bad argument", i);
        if (t.natoms < p.natom_mol || t.natoms % p.natom_mol)
            return cir_fail(CIR_ERR_ARG, "trajectory %d: natoms %d is not a positive multiple of natom_mol %d", i, t.natoms,
                            p.natom_mol);
        const int n = t.natoms / p.natom_mol * p.nchrom_mol;
        if (n > cir_eigh_max_n()) return cir_fail(CIR_ERR_ARG, "trajectory %d: %d chromophores exceed %d", i, n, cir_eigh_max_n());
        if (!t.frame_of_step && t.nframes != steps)
            return cir_fail(CIR_ERR_ARG, "trajectory %d: %d frames for %lld frame-steps", i, t.nframes, steps);
        if (t.frame_of_step)
            for (long long k = 0; k < steps; k++)
                if (t.frame_of_step[k] < 0 || t.frame_of_step[k] >= t.nframes)
                    return cir_fail(CIR_ERR_ARG, "trajectory %d: frame_of_step[%lld] = %d outside [0, %d)", i, k,
                                    t.frame_of_step[k], t.nframes);
        const size_t nx = (size_t)t.nframes * t.natoms * 3;
        if (!is_device_ptr(t.xyz) && !all_finite(t.xyz, nx))
            return cir_fail(CIR_ERR_NONFINITE, "trajectory %d: positions contain NaN or Inf", i);
        if (!is_device_ptr(t.box) && !all_finite(t.box, 3 * (size_t)t.nframes))
            return cir_fail(CIR_ERR_NONFINITE, "trajectory %d: box contains NaN or Inf", i);
        groups[t.natoms].push_back(i);
    }
    // the split-BF16 form runs up to CIR_SPLIT_MAXP size groups jointly (every step one
    // launch per product for all of them); the other forms and options group by group
    const bool joint = joint_enabled() && p.precision == CIR_PREC_BF16X3 && !p.share_frames && !p.propagate_vectors &&
                       groups.size() > 1;
    std::vector<std::vector<int>> batches;   // the group ids (natoms) of each joint run
    if (joint) {
        std::vector<int> keys;
        for (auto &kv : groups) keys.push_back(kv.first);
        for (size_t i = 0; i < keys.size(); i += CIR_SPLIT_MAXP)
            batches.emplace_back(keys.begin() + i, keys.begin() + std::min(keys.size(), i + (size_t)CIR_SPLIT_MAXP));
    }
    for (const auto &bt : batches) {
        while (c->gbuf.size() + 1 < bt.size()) c->gbuf.emplace_back(new DevBuf[B_COUNT]);
        std::vector<std::unique_ptr<GroupJob>> jobs;
        std::vector<std::vector<int>> fidxs(bt.size());
        std::vector<std::vector<cir_result>> rss(bt.size());
        for (size_t gi = 0; gi < bt.size(); gi++) {
            const int natoms = bt[gi];
            const std::vector<int> &ids = groups[natoms];
            DevBuf *buf = gi == 0 ? c->buf : c->gbuf[gi - 1].get();
            Group g;
            g.natoms = natoms;
            g.nmol = natoms / p.natom_mol;
            g.n = g.nmol * p.nchrom_mol;
            g.ld = (g.n + 3) & ~3;
            g.ntraj = (int)ids.size();
            long long nf = 0;
            for (int i : ids) nf += traj[i].nframes;
            CK(buf[B_XYZ].ensure((size_t)nf * natoms * 12));
            CK(buf[B_BOX].ensure((size_t)nf * 12));
            fidxs[gi].resize((size_t)g.ntraj * steps);
            long long off = 0;
            for (int j = 0; j < g.ntraj; j++) {
                const cir_traj_in &t = traj[ids[j]];
                CK(cudaMemcpyAsync(buf[B_XYZ].as<float>() + (size_t)off * natoms * 3, t.xyz,
                                   (size_t)t.nframes * natoms * 12, cudaMemcpyDefault, c->stream));
                CK(cudaMemcpyAsync(buf[B_BOX].as<float>() + (size_t)off * 3, t.box, (size_t)t.nframes * 12,
                                   cudaMemcpyDefault, c->stream));
                for (long long k = 0; k < steps; k++)
                    fidxs[gi][(size_t)j * steps + k] = (int)(off + (t.frame_of_step ? t.frame_of_step[k] : k));
                off += t.nframes;
            }
            rss[gi].resize(g.ntraj);
            for (int j = 0; j < g.ntraj; j++) rss[gi][j] = results[ids[j]];
            jobs.emplace_back(new GroupJob(c, buf, g, buf[B_XYZ].as<float>(), buf[B_BOX].as<float>(), fidxs[gi],
                                           rss[gi].data()));
        }
        const int rc = run_groups_joint(c, jobs);
        if (rc) return rc;
        for (size_t gi = 0; gi < bt.size(); gi++) {
            const std::vector<int> &ids = groups[bt[gi]];
            for (size_t j = 0; j < ids.size(); j++) results[ids[j]] = rss[gi][j];
        }
    }
    for (auto &kv : groups) {
        if (joint) break;
        const int natoms = kv.first;
        const std::vector<int> &ids = kv.second;
        Group g;
        g.natoms = natoms;
        g.nmol = natoms / p.natom_mol;
        g.n = g.nmol * p.nchrom_mol;
        g.ld = (g.n + 3) & ~3;
        g.ntraj = (int)ids.size();
        long long nf = 0;
        for (int i : ids) nf += traj[i].nframes;
        CK(c->buf[B_XYZ].ensure((size_t)nf * natoms * 12));
        CK(c->buf[B_BOX].ensure((size_t)nf * 12));
        std::vector<int> fidx((size_t)g.ntraj * steps);
        long long off = 0;
        for (int j = 0; j < g.ntraj; j++) {
            const cir_traj_in &t = traj[ids[j]];
            CK(cudaMemcpyAsync(c->buf[B_XYZ].as<float>() + (size_t)off * natoms * 3, t.xyz, (size_t)t.nframes * natoms * 12,
                               cudaMemcpyDefault, c->stream));
            CK(cudaMemcpyAsync(c->buf[B_BOX].as<float>() + (size_t)off * 3, t.box, (size_t)t.nframes * 12, cudaMemcpyDefault,
                               c->stream));
            for (long long k = 0; k < steps; k++)
                fidx[(size_t)j * steps + k] = (int)(off + (t.frame_of_step ? t.frame_of_step[k] : k));
            off += t.nframes;
        }
        std::vector<cir_result> rs(g.ntraj);
        for (int j = 0; j < g.ntraj; j++) rs[j] = results[ids[j]];
        const int rc = run_group(c, g, c->buf[B_XYZ].as<float>(), c->buf[B_BOX].as<float>(), fidx, rs.data(), nullptr);
        if (rc) return rc;
        for (int j = 0; j < g.ntraj; j++) results[ids[j]] = rs[j];
    }
    return CIR_OK;
}

// ---------------------------------------------------------------------------------------
// Differentiation form: the gradient of a spectrum-mismatch loss with respect to the map and
// coupling coefficients, by the adjoint of the propagation and of the eigendecomposition.
// ---------------------------------------------------------------------------------------

extern "C" int cir_get_coeffs(cir_ctx *c, float *theta) {
    if (!c || !theta) return cir_fail(CIR_ERR_ARG, "cir_get_coeffs: bad argument");
    const CirMaps &m = c->maps;
    const float v[CIR_NTHETA] = {m.w[0], m.w[1], m.w[2], m.x[0], m.x[1], m.p[0], m.p[1],
                                 m.mup[0], m.mup[1], m.mup[2], m.wi[0], m.wi[1], m.wi[2]};
    memcpy(theta, v, sizeof v);
    return CIR_OK;
}

extern "C" int cir_set_coeffs(cir_ctx *c, const float *t) {
    if (!c || !t) return cir_fail(CIR_ERR_ARG, "cir_set_coeffs: bad argument");
    for (int q = 0; q < CIR_NTHETA; q++)
        if (!std::isfinite(t[q])) return cir_fail(CIR_ERR_NONFINITE, "cir_set_coeffs: coefficient %d is not finite", q);
    CirMaps &m = c->maps;
    m.w[0] = t[0]; m.w[1] = t[1]; m.w[2] = t[2];
    m.x[0] = t[3]; m.x[1] = t[4];
    m.p[0] = t[5]; m.p[1] = t[6];
    m.mup[0] = t[7]; m.mup[1] = t[8]; m.mup[2] = t[9];
    m.wi[0] = t[10]; m.wi[1] = t[11]; m.wi[2] = t[12];
    return CIR_OK;
}

// Positions in the C2R output of the printed lineshape rows (the selection of lineshape_rows),
// and the intensity normalisation.
static std::vector<int> lineshape_index(const cir_params *p, float *norm_out) {
    const int n = p->ntcfpoints + p->nzeros;
    const float factor = (float)(2 * CIR_PI * CIR_HBAR / (p->dt * (float)n));
    *norm_out = factor * (float)n;
    std::vector<int> idx;
    for (int i = n / 2; i < n; i++)
        if (-1 * (i - p->ntcfpoints - p->nzeros) * factor + p->avef <= (float)p->omegaStop) idx.push_back(i);
    for (int i = 0; i < p->ntcfpoints + p->nzeros / 2; i++)
        if (-1 * i * factor + p->avef >= (float)p->omegaStart) idx.push_back(i);
    return idx;
}

// x <- V_k exp(i L_k dt/hbar) V_k^T x for S origins, x n x 9 complex (row-major, 18 floats per
// row); FP32 SIMT GEMMs.  V: origin s at V + s*sV, w likewise; tmp: S x n x 18.
static int psi_propagate(cir_ctx *c, int S, int n, int ld, const float *V, long long sV, const float *w, long long sw,
                         float dt, float *x, float *tmp, int &launches) {
    // X = e^{i L dt/hbar} V^T psi, then psi = V X: two streaming passes over V (k_adjoint.cu)
    CK(cir_psi_step(V, ld, sV, n, w, sw, (float)(dt / CIR_HBAR), x, tmp, S, c->stream));
    launches += 2;
    return CIR_OK;
}

// psi is checkpointed every CKPT steps (psi(0), then psi(j*CKPT - 1)); the backward pass
// recomputes one segment of CKPT steps at a time from its checkpoint.
constexpr int CKPT = 16;

extern "C" int cir_loss_grad(cir_ctx *c, int nframes, const float *xyz, const float *box, const int *frame_of_step,
                             const float *target_ir, const float *target_vv, int nls, double *loss, double *grad) {
    if (!c || !xyz || !box || !target_ir || !target_vv || !loss || !grad || nframes < 1)
        return cir_fail(CIR_ERR_ARG, "cir_loss_grad: bad argument");
    const cir_params &p = c->p;
    const int S = p.nsamples, K = p.ntcfpoints, n = c->n, ld = c->ld;
    const long long steps = (long long)S * K;
    float norm = 0.f;
    const std::vector<int> rows = lineshape_index(&p, &norm);
    if (nls != (int)rows.size())
        return cir_fail(CIR_ERR_ARG, "cir_loss_grad: %d target rows, the lineshape has %zu", nls, rows.size());
    std::vector<int> fidx(steps);
    for (long long i = 0; i < steps; i++) {
        const int f = frame_of_step ? frame_of_step[i] : (int)i;
        if (f < 0 || f >= nframes) return cir_fail(CIR_ERR_ARG, "frame_of_step[%lld] = %d outside [0, %d)", i, f, nframes);
        fidx[i] = f;
    }
    const size_t nx = (size_t)nframes * c->natoms * 3;
    if (!is_device_ptr(xyz) && !all_finite(xyz, nx)) return cir_fail(CIR_ERR_NONFINITE, "positions contain NaN or Inf");
    if (!is_device_ptr(box) && !all_finite(box, 3 * (size_t)nframes)) return cir_fail(CIR_ERR_NONFINITE, "box contains NaN or Inf");
    // every frame-step of the job stays resident (one chunk)
    const long long mstride = (long long)n * ld;
    const size_t per_step = (size_t)2 * mstride * 4 + cir_dc_bytes(n, ld) + cir_eigh_de_bytes(ld) +
                            (size_t)(9 + CT_NROW + 1) * ld * 4 + (size_t)c->natoms * 12 + 64;
    size_t freeb = 0, totalb = 0;
    if (cudaMemGetInfo(&freeb, &totalb) == cudaSuccess && per_step * steps > freeb / 2)
        return cir_fail(CIR_ERR_NOMEM, "cir_loss_grad: %lld frame-steps need %.1f GB (half the free memory: %.1f GB)",
                        steps, per_step * steps / 1e9, freeb / 2e9);
    if (steps > 65535) return cir_fail(CIR_ERR_ARG, "cir_loss_grad: %lld frame-steps (at most 65535)", steps);
    void *dxyz, *dbox;
    int rc;
    if ((rc = stage_in(c, B_XYZ, xyz, nx * 4, &dxyz, true))) return rc;
    if ((rc = stage_in(c, B_BOX, box, (size_t)nframes * 12, &dbox, true))) return rc;
    const int nb = (int)steps;
    const size_t psz = (size_t)S * n * CIR_PSI_LD;            // floats of one psi set
    const int nseg = (K + CKPT - 1) / CKPT;
    CK(c->buf[B_FIDX].ensure((size_t)steps * 4));
    CK(cudaMemcpyAsync(c->buf[B_FIDX].p, fidx.data(), (size_t)steps * 4, cudaMemcpyHostToDevice, c->stream));
    CK(c->buf[B_CXYZ].ensure((size_t)nb * c->natoms * 12));
    CK(c->buf[B_CBOX].ensure((size_t)nb * 12));
    CK(c->buf[B_CT].ensure((size_t)nb * CT_NROW * ld * 4));
    CK(c->buf[B_A].ensure((size_t)nb * mstride * 4));
    CK(c->buf[B_Z].ensure((size_t)nb * mstride * 4));
    CK(c->buf[B_DC].ensure((size_t)nb * cir_dc_bytes(n, ld)));
    CK(c->buf[B_DE].ensure((size_t)nb * cir_eigh_de_bytes(ld)));
    CK(c->buf[B_W].ensure((size_t)nb * ld * 4));
    CK(c->buf[B_M].ensure((size_t)nb * 9 * ld * 4));
    CK(c->buf[B_STATUS].ensure((size_t)nb * 4));
    CK(c->buf[B_PSI].ensure(psz * 4));
    CK(c->buf[B_LAM].ensure(psz * 4));
    CK(c->buf[B_PA].ensure(psz * 4));
    CK(c->buf[B_PB].ensure(psz * 4));
    CK(c->buf[B_SEG].ensure(psz * (CKPT + 1) * 4));
    CK(c->buf[B_CKPT].ensure(psz * nseg * 4));
    CK(c->buf[B_R].ensure((size_t)S * mstride * 4));
    CK(c->buf[B_T].ensure((size_t)S * mstride * 4));
    CK(c->buf[B_TCF].ensure((size_t)steps * 48));
    CK(c->buf[B_GRAD].ensure(CIR_NTHETA * 8));
    CK(cudaMemsetAsync(c->buf[B_STATUS].p, 0, (size_t)nb * 4, c->stream));
    CK(cudaMemsetAsync(c->buf[B_GRAD].p, 0, CIR_NTHETA * 8, c->stream));
    float *A = c->buf[B_A].as<float>(), *W = c->buf[B_W].as<float>(), *M = c->buf[B_M].as<float>();
    float *CT = c->buf[B_CT].as<float>(), *CB = c->buf[B_CBOX].as<float>();
    float *psi = c->buf[B_PSI].as<float>(), *lam = c->buf[B_LAM].as<float>();
    float *PA = c->buf[B_PA].as<float>(), *PB = c->buf[B_PB].as<float>();
    float *seg = c->buf[B_SEG].as<float>(), *ckpt = c->buf[B_CKPT].as<float>();
    float *R = c->buf[B_R].as<float>(), *T = c->buf[B_T].as<float>();
    double *tcf = c->buf[B_TCF].as<double>(), *dgrad = c->buf[B_GRAD].as<double>();
    int launches = 0;
    // frames, Hamiltonians and eigendecompositions of every step (origin-major: b = s*K + k)
    Group g = ctx_group(c);
    k_gather_frames<<<dim3(8, nb), 256, 0, c->stream>>>(static_cast<const float *>(dxyz), static_cast<const float *>(dbox),
                                                        c->buf[B_FIDX].as<int>(), g.natoms, S, K, K, 0,
                                                        c->buf[B_CXYZ].as<float>(), CB);
    CK(cudaGetLastError());
    launches++;
    BuildArgs ba = build_args(c, g);
    ba.xyz = c->buf[B_CXYZ].as<float>();
    ba.box = CB;
    ba.ct = CT;
    ba.H = A;
    ba.ldh = ld;
    ba.dip = M;
    ba.pol = M + 3 * ld;
    ba.ldv = ld;
    ba.dip_fstride = 9LL * ld;
    ba.pol_fstride = 9LL * ld;
    CK(cir_launch_build(ba, nb, c->stream, &launches));
    EighArgs e;
    memset(&e, 0, sizeof e);
    e.A = A;
    e.W = W;
    e.Z = c->buf[B_Z].as<float>();
    e.DC = c->buf[B_DC].as<float>();
    e.DE = c->buf[B_DE].as<float>();
    e.mstride = mstride;
    e.wstride = ld;
    e.n = n;
    e.ld = ld;
    e.status = c->buf[B_STATUS].as<int>();
    e.nchrom_mol = p.nchrom_mol;
    e.precision = CIR_PREC_FP32;
    e.err = c->buf[B_ERR].as<int>();
    e.test_stall = c->p.test_stall_gemm;
    e.test_sweep_cap = c->p.test_sweep_cap;
    CK(cir_launch_eigh(e, nb, c->stream, &launches));
    // forward: psi(0) = m(0); psi(k) = U_k psi(k-1); correlation terms per step; checkpoints
    const long long sV = (long long)K * mstride, sWk = (long long)K * ld, sM = (long long)K * 9 * ld;
    CK(cir_adj_psi_init(M, sM, ld, n, S, psi, c->stream));
    launches++;
    for (int k = 0; k < K; k++) {
        if (k > 0 && (rc = psi_propagate(c, S, n, ld, A + (size_t)k * mstride, sV, W + (size_t)k * ld, sWk, p.dt, psi, PA,
                                         launches)))
            return rc;
        CK(cir_adj_tcf(psi, M + (size_t)k * 9 * ld, sM, ld, n, S, tcf + (size_t)k * 6, (long long)K * 6, c->stream));
        launches++;
        if (k == 0 || (k + 1) % CKPT == 0) {
            const int slot = k == 0 ? 0 : (k + 1) / CKPT;
            if (slot < nseg) CK(cudaMemcpyAsync(ckpt + psz * slot, psi, psz * 4, cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    // loss: lineshapes of the damped, origin-averaged IR and VV sums against the targets
    std::vector<double> htcf((size_t)steps * 6);
    std::vector<int> hst(nb);
    CK(cudaMemcpyAsync(htcf.data(), tcf, (size_t)steps * 48, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(hst.data(), c->buf[B_STATUS].p, (size_t)nb * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nb; i++)
        if (hst[i]) return cir_fail(CIR_ERR_NOCONVERGE, "eigensolver sweep cap reached");
    std::vector<double> dcy(K), X[2];
    for (int q = 0; q < 2; q++) X[q].assign((size_t)2 * K, 0.0);
    for (int k = 0; k < K; k++) {
        dcy[k] = exp(-1.0 * k * p.dt / (2.0 * p.t1)) / (1. * S);
        CompSum sum[4];                              // IR (terms 0, 1) and VV (terms 2, 3)
        for (int s = 0; s < S; s++)
            for (int q = 0; q < 4; q++) sum[q].add(htcf[((size_t)s * K + k) * 6 + q]);
        for (int q = 0; q < 2; q++) {
            X[q][2 * k] = sum[2 * q].value() * dcy[k];
            X[q][2 * k + 1] = sum[2 * q + 1].value() * dcy[k];
        }
    }
    const int nfft = p.ntcfpoints + p.nzeros;
    const float *tg[2] = {target_ir, target_vv};
    double L = 0.0;
    std::vector<double> gre[2], gim[2];
    for (int q = 0; q < 2; q++) {
        std::vector<double> y;
        if ((rc = c2r_dev(c, X[q].data(), y))) return rc;
        gre[q].assign(K, 0.0);
        gim[q].assign(K, 0.0);
        // dL/dX_k = sum over rows of dL/dy_i dy_i/dX_k; y_i = Re X_0 + 2 sum_k Re(X_k e^{2 pi i ik/n})
        for (size_t r = 0; r < rows.size(); r++) {
            const int i = rows[r];
            const double ls = (float)y[i] / norm;      // the printed value, as lineshape_rows makes it
            const double d = ls - tg[q][r];
            L += d * d;
            const double dy = 2.0 * d / norm;
            gre[q][0] += dy;
            for (int k = 1; k < K; k++) {
                const double ang = 2.0 * CIR_PI * (double)((long long)i * k % nfft) / nfft;
                gre[q][k] += 2.0 * dy * cos(ang);
                gim[q][k] -= 2.0 * dy * sin(ang);
            }
        }
        for (int k = 0; k < K; k++) {              // through the damping and 1/nsamples
            gre[q][k] *= dcy[k];
            gim[q][k] *= dcy[k];
        }
    }
    // backward, one segment of CKPT steps at a time, last segment first
    const float tau = (float)(p.dt / CIR_HBAR);
    DthetaArgs dt{};
    dt.sct = (long long)K * CT_NROW * ld;
    dt.sbox = 3LL * K;
    dt.ldg = ld;
    dt.sG = mstride;
    dt.maps = c->maps;
    dt.n = n;
    dt.ld = ld;
    dt.nchrom_mol = p.nchrom_mol;
    dt.ispecies = p.ispecies;
    dt.out = dgrad;
    for (int j = nseg - 1; j >= 0; j--) {
        const int c0 = j * CKPT, c1 = std::min(K, c0 + CKPT);
        const int base = c0 == 0 ? 0 : c0 - 1;        // seg slot q holds psi(base + q)
        CK(cudaMemcpyAsync(seg, ckpt + psz * j, psz * 4, cudaMemcpyDeviceToDevice, c->stream));
        for (int k = base + 1; k < c1; k++) {
            float *dst = seg + psz * (k - base);
            CK(cudaMemcpyAsync(dst, seg + psz * (k - 1 - base), psz * 4, cudaMemcpyDeviceToDevice, c->stream));
            if ((rc = psi_propagate(c, S, n, ld, A + (size_t)k * mstride, sV, W + (size_t)k * ld, sWk, p.dt, dst, PA,
                                    launches)))
                return rc;
        }
        for (int k = c1 - 1; k >= c0; k--) {
            // lambda(k) = w(k) + U_{k+1} lambda(k+1)
            if (k < K - 1 && (rc = psi_propagate(c, S, n, ld, A + (size_t)(k + 1) * mstride, sV, W + (size_t)(k + 1) * ld,
                                                 sWk, p.dt, lam, PA, launches)))
                return rc;
            CK(cir_adj_lambda_src(lam, M + (size_t)k * 9 * ld, sM, ld, n, S, (float)gre[0][k], (float)gim[0][k],
                                  (float)gre[1][k], (float)gim[1][k], k == K - 1, c->stream));
            launches++;
            const float *Vk = A + (size_t)k * mstride;
            if (k >= 1) {
                // a = V^T lambda(k), b = V^T psi(k-1); R; G = V R V^T (into R)
                GemmArgs ga{};
                ga.A = Vk; ga.lda = ld; ga.sA = sV; ga.a_colmajor = false;
                ga.B = lam; ga.ldb = CIR_PSI_LD; ga.sB = (long long)n * CIR_PSI_LD;
                ga.C = PA; ga.ldc = CIR_PSI_LD; ga.sC = (long long)n * CIR_PSI_LD;
                ga.M = n; ga.N = CIR_PSI_LD; ga.K = n;
                GemmArgs gb = ga;
                gb.B = seg + psz * (k - 1 - base);
                gb.C = PB;
                CK(cir_launch_gemm(ga, S, c->stream, &launches));
                CK(cir_launch_gemm(gb, S, c->stream, &launches));
                CK(cir_adj_build_R(PA, PB, W + (size_t)k * ld, sWk, n, S, tau, R, ld, mstride, c->stream));
                launches++;
                GemmArgs gt{};
                gt.A = Vk; gt.lda = ld; gt.sA = sV; gt.a_colmajor = true;     // V
                gt.B = R; gt.ldb = ld; gt.sB = mstride;                        // R row-major
                gt.C = T; gt.ldc = ld; gt.sC = mstride;
                gt.M = gt.N = gt.K = n;
                GemmArgs gg = gt;
                gg.A = T; gg.a_colmajor = false; gg.sA = mstride;              // T row-major
                gg.B = Vk; gg.sB = sV;                                         // B(k, j) = V[j][k]
                gg.C = R;
                CK(cir_launch_gemm(gt, S, c->stream, &launches));
                CK(cir_launch_gemm(gg, S, c->stream, &launches));
            }
            dt.ct = CT + (size_t)k * CT_NROW * ld;
            dt.box = CB + 3 * (size_t)k;
            dt.G = k >= 1 ? R : nullptr;
            dt.psi = seg + psz * (k - base);
            dt.lam0 = k == 0 ? lam : nullptr;
            dt.gir_r = (float)gre[0][k];
            dt.gir_i = (float)gim[0][k];
            dt.gvv_r = (float)gre[1][k];
            dt.gvv_i = (float)gim[1][k];
            CK(cir_adj_dtheta(dt, S, c->stream));
            launches++;
        }
    }
    CK(cudaMemcpyAsync(grad, dgrad, CIR_NTHETA * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    count_launch(c, launches);
    *loss = L;
    return CIR_OK;
}
