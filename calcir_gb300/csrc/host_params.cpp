// Run parameters: defaults, the input.inp parser, decoding and the output writers.
// The parser keeps the token semantics of the reference's ir_init
// (calcIR.cu:1539-1643): fscanf("%s%s%*[^\n]") reads a key and a value token,
// either of which may sit on a later line, and drops the rest of the line.
#include "cir_internal.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

static thread_local char g_err[1024];

extern "C" int cir_fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

extern "C" const char *cir_last_error(void) { return g_err; }
extern "C" const char *cir_version(void) { return CIR_VERSION_STRING; }

bool cir_maps(int imap, int ispecies, CirMaps *m) {
    const bool h = (ispecies == 0 || ispecies == 1);   // H2O, HOD/D2O: OH stretch maps
    if (imap == 0) {                                     // Gruenbaum et al. 2013
        if (h) { m->w[0] = 3670.2f; m->w[1] = -3541.7f; m->w[2] = -152677.0f;
                 m->x[0] = 0.19285f; m->x[1] = -1.7261E-5f; m->p[0] = 1.6466f; m->p[1] = 5.7692E-4f; }
        else   { m->w[0] = 2767.8f; m->w[1] = -2630.3f; m->w[2] = -102601.0f;
                 m->x[0] = 0.16593f; m->x[1] = -2.0632E-5f; m->p[0] = 2.0475f; m->p[1] = 8.9108E-4f; }
        m->mup[0] = 0.1646f; m->mup[1] = 11.39f; m->mup[2] = 63.41f;
        m->wi[0] = -1361.0f; m->wi[1] = 27165.0f; m->wi[2] = -1.887f;
        return true;
    }
    if (imap == 1) {                                     // Li and Skinner 2010
        if (h) { m->w[0] = 3732.9f; m->w[1] = -3519.8f; m->w[2] = -153520.0f;
                 m->x[0] = 0.19318f; m->x[1] = -1.7248E-5f; m->p[0] = 1.6102f; m->p[1] = 5.8697E-4f; }
        else   { m->w[0] = 2748.2f; m->w[1] = -2572.2f; m->w[2] = -102980.0f;
                 m->x[0] = 0.16598f; m->x[1] = -2.0752E-5f; m->p[0] = 1.9813f; m->p[1] = 9.1419E-4f; }
        m->mup[0] = 0.1622f; m->mup[1] = 10.381f; m->mup[2] = 137.6f;
        m->wi[0] = -1360.8f; m->wi[1] = 27171.0f; m->wi[2] = -1.887f;
        return true;
    }
    return false;
}

static void set_str(char *dst, const char *src) {
    strncpy(dst, src, CIR_STRLEN - 1);
    dst[CIR_STRLEN - 1] = 0;
}

extern "C" int cir_params_default(cir_params *p) {
    if (!p) return cir_fail(CIR_ERR_ARG, "cir_params_default: null pointer");
    memset(p, 0, sizeof *p);
    set_str(p->xtcf, "traj.xtc");
    set_str(p->outf, "spec");
    set_str(p->cptf, "spec");
    set_str(p->model, "e3b3");
    set_str(p->species, " ");       // the reference default, which its decoder rejects
    p->ntcfpoints = 150;
    p->nsamples = 1;
    p->sampleEvery = 10.f;
    p->omegaStart = 2000;
    p->omegaStop = 5000;
    p->omegaStep = 5;
    p->natom_mol = 4;
    p->nchrom_mol = 2;
    p->nzeros = 25600;
    p->dt = 0.010f;
    p->beginTime = 0;
    p->t1 = 0.260f;
    p->avef = 3415.2f;
    p->map = 0;
    p->imodel = 0;
    p->ispecies = 0;
    p->synth_nmol = 64;
    p->synth_seed = 1;
    p->synth_frame_dt = 0.010f;
    p->synth_sigma_trans = 0.003f;
    p->synth_sigma_rot = 3.0f;
    p->precision = CIR_PREC_FP32;
    p->batch_frames = 0;
    p->verbose = 0;
    p->cuda_graphs = 1;
    p->autotune = 1;
    p->propagate_vectors = 0;
    p->share_frames = 0;
    p->refine_eigen = 0;
    return CIR_OK;
}

// sscanf(value, "%d", &x): a leading integer, or no assignment.
static void scan_int(const char *v, int *x) {
    char *end = nullptr;
    long r = strtol(v, &end, 10);
    if (end != v) *x = (int)r;
}
// sscanf(value, "%f", &x): a leading float, or no assignment.
static void scan_float(const char *v, float *x) {
    char *end = nullptr;
    float r = strtof(v, &end);
    if (end != v) *x = r;
}

// Reads one whitespace-delimited token; false at end of file.
static bool read_token(FILE *f, std::string &tok) {
    int ch;
    do { ch = fgetc(f); } while (ch != EOF && isspace(ch));
    if (ch == EOF) return false;
    tok.clear();
    while (ch != EOF && !isspace(ch)) { tok.push_back((char)ch); ch = fgetc(f); }
    if (ch != EOF) ungetc(ch, f);
    return true;
}

extern "C" int cir_params_parse_file(const char *path, cir_params *p) {
    if (!path || !p) return cir_fail(CIR_ERR_ARG, "cir_params_parse_file: null pointer");
    FILE *f = fopen(path, "r");
    if (!f)
        return cir_fail(CIR_ERR_IO,
                        "ERROR: Could not open %s. The first argument should contain  a  vaild\n"
                        "file name that points to a file containing the simulation parameters.",
                        path);
    if (p->verbose) printf(">>> Reading parameters from input file %s\n", path);
    std::string para, value;   // value keeps its content when a line lacks one, as in C
    while (read_token(f, para)) {
        read_token(f, value);
        // %*[^\n]: drop the rest of the line
        int ch;
        while ((ch = fgetc(f)) != EOF && ch != '\n') {}
        if (ch == '\n') ungetc(ch, f);
        if (para.size() >= CIR_STRLEN || value.size() >= CIR_STRLEN) {
            fclose(f);
            return cir_fail(CIR_ERR_PARSE, "input token longer than %d characters", CIR_STRLEN - 1);
        }
        const char *k = para.c_str(), *v = value.c_str();
        if (!strcmp(k, "xtcf")) set_str(p->xtcf, v);
        else if (!strcmp(k, "outf")) set_str(p->outf, v);
        else if (!strcmp(k, "cptf")) set_str(p->cptf, v);
        else if (!strcmp(k, "model")) set_str(p->model, v);
        else if (!strcmp(k, "ntcfpoints")) scan_int(v, &p->ntcfpoints);
        else if (!strcmp(k, "nsamples")) scan_int(v, &p->nsamples);
        else if (!strcmp(k, "sampleEvery")) scan_float(v, &p->sampleEvery);
        else if (!strcmp(k, "omegaStep")) scan_int(v, &p->omegaStep);
        else if (!strcmp(k, "natom_mol")) scan_int(v, &p->natom_mol);
        else if (!strcmp(k, "nchrom_mol")) scan_int(v, &p->nchrom_mol);
        else if (!strcmp(k, "nzeros")) scan_int(v, &p->nzeros);
        else if (!strcmp(k, "map")) scan_int(v, &p->map);
        else if (!strcmp(k, "species")) set_str(p->species, v);
        else if (!strcmp(k, "dt")) scan_float(v, &p->dt);
        else if (!strcmp(k, "t1")) scan_float(v, &p->t1);
        else if (!strcmp(k, "avef")) scan_float(v, &p->avef);
        else if (!strcmp(k, "beginTime")) scan_float(v, &p->beginTime);
        else if (!strcmp(k, "omegaStart")) scan_float(v, &p->omegaStart);
        else if (!strcmp(k, "omegaStop")) scan_float(v, &p->omegaStop);
        // keys added by this implementation
        else if (!strcmp(k, "synth_nmol")) scan_int(v, &p->synth_nmol);
        else if (!strcmp(k, "synth_seed")) scan_int(v, &p->synth_seed);
        else if (!strcmp(k, "synth_frame_dt")) scan_float(v, &p->synth_frame_dt);
        else if (!strcmp(k, "synth_sigma_trans")) scan_float(v, &p->synth_sigma_trans);
        else if (!strcmp(k, "synth_sigma_rot")) scan_float(v, &p->synth_sigma_rot);
        else if (!strcmp(k, "batch_frames")) scan_int(v, &p->batch_frames);
        else if (!strcmp(k, "verbose")) scan_int(v, &p->verbose);
        else if (!strcmp(k, "cuda_graphs")) scan_int(v, &p->cuda_graphs);
        else if (!strcmp(k, "autotune")) scan_int(v, &p->autotune);
        else if (!strcmp(k, "propagate_vectors")) scan_int(v, &p->propagate_vectors);
        else if (!strcmp(k, "share_frames")) scan_int(v, &p->share_frames);
        else if (!strcmp(k, "refine_eigen")) scan_int(v, &p->refine_eigen);
        else if (!strcmp(k, "precision")) {
            if (!strcmp(v, "fp32")) p->precision = CIR_PREC_FP32;
            else if (!strcmp(v, "tf32")) p->precision = CIR_PREC_TF32;
            else if (!strcmp(v, "bf16x3")) p->precision = CIR_PREC_BF16X3;
            else { fclose(f); return cir_fail(CIR_ERR_PARSE, "precision %s is not one of fp32, tf32, bf16x3", v); }
        } else {
            printf("WARNING: Parameter %s in input file %s not recognized, ignoring.\n", k, path);
        }
    }
    fclose(f);
    if (p->verbose) printf(">>> Done reading input file and setting parameters\n");
    fflush(stdout);
    return CIR_OK;
}

extern "C" int cir_params_finalize(cir_params *p) {
    if (!p) return cir_fail(CIR_ERR_ARG, "cir_params_finalize: null pointer");
    // calcIR.cu:325-330
    if (!strcmp(p->model, "tip4p2005") || !strcmp(p->model, "e3b3")) p->imodel = 1;
    else if (!strcmp(p->model, "tip4p") || !strcmp(p->model, "e3b2")) p->imodel = 0;
    else return cir_fail(CIR_ERR_PARSE, "WARNING: model: %s is not recognized. Check input file. Aborting...", p->model);
    // calcIR.cu:332-339
    if (!strcmp(p->species, "H2O")) p->ispecies = 0;
    else if (!strcmp(p->species, "HOD/D2O")) p->ispecies = 1;
    else if (!strcmp(p->species, "HOD/H2O")) p->ispecies = 2;
    else if (!strcmp(p->species, "D2O")) p->ispecies = 3;
    else return cir_fail(CIR_ERR_PARSE, "WARNING: species: %s is not recognized. Check input file. Aborting...", p->species);
    // other map values leave the reference's map arrays uninitialised (calcIR.cu:1207-1242)
    if (p->map != 0 && p->map != 1) return cir_fail(CIR_ERR_PARSE, "map %d is not 0 or 1", p->map);
    if (p->ntcfpoints < 1 || p->nsamples < 1) return cir_fail(CIR_ERR_ARG, "ntcfpoints and nsamples must be >= 1");
    if (p->omegaStep < 1) return cir_fail(CIR_ERR_ARG, "omegaStep must be >= 1");
    if (p->nzeros < 0) return cir_fail(CIR_ERR_ARG, "nzeros must be >= 0");
    if (p->ntcfpoints + p->nzeros < 2) return cir_fail(CIR_ERR_ARG, "ntcfpoints + nzeros must be >= 2");
    if (!(p->dt > 0) || !(p->t1 > 0)) return cir_fail(CIR_ERR_ARG, "dt and t1 must be > 0");
    if (p->natom_mol < 3 || p->natom_mol > 64) return cir_fail(CIR_ERR_ARG, "natom_mol must be in [3, 64]");
    if (p->nchrom_mol < 1 || p->nchrom_mol > 2) return cir_fail(CIR_ERR_ARG, "nchrom_mol must be 1 or 2");
    if (cir_nomega(p) < 1) return cir_fail(CIR_ERR_ARG, "omegaStop must not be below omegaStart");
    if (p->precision < CIR_PREC_FP32 || p->precision > CIR_PREC_BF16X3)
        return cir_fail(CIR_ERR_ARG, "precision %d unknown", p->precision);
    if (p->refine_eigen < 0 || p->refine_eigen > 8)
        return cir_fail(CIR_ERR_ARG, "refine_eigen must be in [0, 8] (refinement steps)");
    return CIR_OK;
}

extern "C" int cir_nomega(const cir_params *p) {
    // float arithmetic truncated to int, calcIR.cu:94
    return (int)((p->omegaStop - p->omegaStart) / p->omegaStep + 1);
}

// Conversion factor of the lineshape axis: double arithmetic stored to float (calcIR.cu:890).
static float ls_factor(const cir_params *p) {
    return (float)(2 * CIR_PI * CIR_HBAR / (p->dt * (float)(p->ntcfpoints + p->nzeros)));
}

extern "C" int cir_result_sizes(const cir_params *p, int *ntcf, int *nomega, int *nls) {
    if (!p) return cir_fail(CIR_ERR_ARG, "cir_result_sizes: null pointer");
    if (ntcf) *ntcf = p->ntcfpoints;
    if (nomega) *nomega = cir_nomega(p);
    if (nls) {
        const int n = p->ntcfpoints + p->nzeros;
        const float factor = ls_factor(p);
        int cnt = 0;
        for (int i = n / 2; i < n; i++) {
            float freq = -1 * (i - p->ntcfpoints - p->nzeros) * factor + p->avef;
            if (freq <= (float)p->omegaStop) cnt++;
        }
        for (int i = 0; i < p->ntcfpoints + p->nzeros / 2; i++) {
            float freq = -1 * i * factor + p->avef;
            if (freq >= (float)p->omegaStart) cnt++;
        }
        *nls = cnt;
    }
    return CIR_OK;
}

extern "C" int cir_frame_index(const cir_params *p, float frame_dt, int sample, int step, int *frame) {
    if (!p || !frame || !(frame_dt > 0)) return cir_fail(CIR_ERR_ARG, "cir_frame_index: bad argument");
    // float arithmetic in the reference's order, calcIR.cu:378-379
    float desired_time = sample * p->sampleEvery + p->beginTime + p->dt * step;
    *frame = (int)roundf(desired_time / frame_dt);
    return CIR_OK;
}

static FILE *open_out(const cir_params *p, const char *suffix) {
    std::string name = std::string(p->outf) + suffix;
    return fopen(name.c_str(), "w");
}

extern "C" int cir_write_outputs(const cir_params *p, const cir_result *r) {
    if (!p || !r) return cir_fail(CIR_ERR_ARG, "cir_write_outputs: null pointer");
    const int ntcf = p->ntcfpoints, nomega = cir_nomega(p);
    // time correlation functions, "%g %g \n" (calcIR.cu:844-866)
    const char *tsuf[6] = {"_irrtcf.dat", "_iritcf.dat", "_vvrtcf.dat", "_vvitcf.dat", "_vhrtcf.dat", "_vhitcf.dat"};
    const double *tsrc[3] = {r->tcf_ir, r->tcf_vv, r->tcf_vh};
    for (int f = 0; f < 6; f++) {
        FILE *o = open_out(p, tsuf[f]);
        if (!o) return cir_fail(CIR_ERR_IO, "cannot write %s%s", p->outf, tsuf[f]);
        for (int i = 0; i < ntcf; i++)
            fprintf(o, "%g %g \n", (double)(i * p->dt), (double)(float)tsrc[f / 2][2 * i + (f & 1)]);
        fclose(o);
    }
    // spectral density and frequency distributions, "%g %g\n" (calcIR.cu:870-886)
    const char *wsuf[4] = {"_spdn.dat", "_Pw.dat", "_Rw.dat", "_Rmw.dat"};
    const float *wsrc[4] = {r->sw, r->pw, r->rw, r->rmw};
    for (int f = 0; f < 4; f++) {
        FILE *o = open_out(p, wsuf[f]);
        if (!o) return cir_fail(CIR_ERR_IO, "cannot write %s%s", p->outf, wsuf[f]);
        for (int i = 0; i < nomega; i++) fprintf(o, "%g %g\n", (double)r->omega[i], (double)wsrc[f][i]);
        fclose(o);
    }
    // lineshapes (calcIR.cu:893-919)
    const char *lsuf[3] = {"_irls.dat", "_vvls.dat", "_vhls.dat"};
    const float *lsrc[3] = {r->ls_ir, r->ls_vv, r->ls_vh};
    for (int f = 0; f < 3; f++) {
        FILE *o = open_out(p, lsuf[f]);
        if (!o) return cir_fail(CIR_ERR_IO, "cannot write %s%s", p->outf, lsuf[f]);
        for (int i = 0; i < r->nls; i++) fprintf(o, "%g %g\n", (double)r->ls_omega[i], (double)lsrc[f][i]);
        fclose(o);
    }
    return CIR_OK;
}
