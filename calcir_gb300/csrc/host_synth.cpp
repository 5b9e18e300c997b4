// Seeded synthetic water boxes: the frame source that stands in for a GROMACS .xtc
// trajectory (the reference reads one with libxdrfile, calcIR.cu:212-223, 341-398).
//
// Rigid TIP4P/2005 geometry (O-H 0.09572 nm, HOH 104.52 deg, M 0.01546 nm along the
// bisector), atoms written O, H1, H2, M per molecule.  Frame 0 puts O on a jittered
// simple-cubic lattice with uniformly random orientations; every later frame moves
// each molecule by a Gaussian translation and a small rotation about a random axis,
// redrawing any move that brings an O or H within `min_contact` of another molecule's
// O or H.
//
// Determinism: every random draw is a hash of (seed, frame, molecule, attempt, k), and
// the arithmetic uses only +, -, *, / and sqrt in double precision (this file is built
// with -ffp-contract=off), so x86-64 and aarch64 produce bit-identical frames.
// Gaussian draws are Irwin-Hall sums of 12 uniforms; a rotation by angle a about the
// unit axis u is the unit quaternion proportional to (1, u*a/2).
#include "cir_internal.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Stream {
    uint64_t base;
    uint64_t k = 0;
    Stream(uint64_t seed, uint64_t frame, uint64_t mol, uint64_t attempt)
        : base(mix64(seed ^ mix64(frame ^ mix64(mol ^ mix64(attempt ^ 0x5851F42D4C957F2Dull))))) {}
    double uniform() { return (double)(mix64(base + 0xD1B54A32D192ED03ull * (++k)) >> 11) * 0x1.0p-53; }
    double gauss() {
        double s = 0;
        for (int i = 0; i < 12; i++) s += uniform();
        return s - 6.0;
    }
    // uniform on the unit sphere by rejection from the cube
    void unit3(double u[3]) {
        for (;;) {
            double a = 2 * uniform() - 1, b = 2 * uniform() - 1, c = 2 * uniform() - 1;
            double r2 = a * a + b * b + c * c;
            if (r2 > 1e-4 && r2 <= 1.0) {
                double r = sqrt(r2);
                u[0] = a / r; u[1] = b / r; u[2] = c / r;
                return;
            }
        }
    }
    // uniform on SO(3): a unit quaternion uniform on S^3, by rejection from the 4-cube
    void quat(double q[4]) {
        for (;;) {
            double a = 2 * uniform() - 1, b = 2 * uniform() - 1, c = 2 * uniform() - 1, d = 2 * uniform() - 1;
            double r2 = a * a + b * b + c * c + d * d;
            if (r2 > 1e-4 && r2 <= 1.0) {
                double r = sqrt(r2);
                q[0] = a / r; q[1] = b / r; q[2] = c / r; q[3] = d / r;
                return;
            }
        }
    }
};

// body frame: O at the origin, bisector along +z, molecule in the xz plane
const double R_OH = 0.09572;
const double SIN_HALF = 0.790796413773152;    // sin(104.52 deg / 2)
const double COS_HALF = 0.6120792693463173;   // cos(104.52 deg / 2)
const double D_OM = 0.01546;
const double BODY[4][3] = {{0, 0, 0},
                           {R_OH * SIN_HALF, 0, R_OH * COS_HALF},
                           {-R_OH * SIN_HALF, 0, R_OH * COS_HALF},
                           {0, 0, D_OM}};

void rotmat(const double q[4], double R[3][3]) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - w * z);     R[0][2] = 2 * (x * z + w * y);
    R[1][0] = 2 * (x * y + w * z);     R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - w * x);
    R[2][0] = 2 * (x * z - w * y);     R[2][1] = 2 * (y * z + w * x);     R[2][2] = 1 - 2 * (x * x + y * y);
}

void qmul(const double a[4], const double b[4], double o[4]) {
    o[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    o[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
    o[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
    o[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}

void qnorm(double q[4]) {
    double r = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int i = 0; i < 4; i++) q[i] /= r;
}

double cube_root(double x) {   // Newton iteration with a fixed count: platform independent
    double y = x > 1 ? x / 3 + 0.5 : 1.0;
    for (int i = 0; i < 200; i++) y = y - (y * y * y - x) / (3 * y * y);
    return y;
}

inline double wrap(double v, double L) {
    double f = v / L;
    double fl = (double)(long long)f;
    if (fl > f) fl -= 1;                 // floor
    return v - L * fl;
}

inline double mi(double d, double L) {  // minimum image, round half away from zero
    double f = d / L;
    double r = (double)(long long)(f + (f >= 0 ? 0.5 : -0.5));
    return d - L * r;
}

struct Mol {
    double o[3];
    double q[4];
    double site[3][3];   // O, H1, H2 absolute positions (for contact checks)
};

void place(Mol &m) {
    double R[3][3];
    rotmat(m.q, R);
    for (int s = 0; s < 3; s++)
        for (int a = 0; a < 3; a++)
            m.site[s][a] = m.o[a] + R[a][0] * BODY[s][0] + R[a][1] * BODY[s][1] + R[a][2] * BODY[s][2];
}

struct Box {
    double L;
    int nc;                      // cells per edge (0: no cell list)
    std::vector<int> cell_of;
    std::vector<std::vector<int>> members;
    int cell_index(const double o[3]) const {
        int c[3];
        for (int a = 0; a < 3; a++) {
            int v = (int)(wrap(o[a], L) / L * nc);
            if (v >= nc) v = nc - 1;
            if (v < 0) v = 0;
            c[a] = v;
        }
        return (c[2] * nc + c[1]) * nc + c[0];
    }
};

bool clash_pair(const Mol &a, const Mol &b, double L, double rmin2) {
    for (int s = 0; s < 3; s++)
        for (int t = 0; t < 3; t++) {
            double dx = mi(a.site[s][0] - b.site[t][0], L);
            double dy = mi(a.site[s][1] - b.site[t][1], L);
            double dz = mi(a.site[s][2] - b.site[t][2], L);
            if (dx * dx + dy * dy + dz * dz < rmin2) return true;
        }
    return false;
}

// any clash between candidate `m` (index j) and molecules other than j; `placed` limits
// the check to molecules [0, placed) during the initial build
bool clashes(const Mol &m, int j, const std::vector<Mol> &mols, int placed, const Box &bx, double rmin2) {
    if (bx.nc >= 3) {
        int cc = bx.cell_index(m.o);
        int cx = cc % bx.nc, cy = (cc / bx.nc) % bx.nc, cz = cc / (bx.nc * bx.nc);
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int x = (cx + dx + bx.nc) % bx.nc, y = (cy + dy + bx.nc) % bx.nc, z = (cz + dz + bx.nc) % bx.nc;
                    for (int k : bx.members[(z * bx.nc + y) * bx.nc + x]) {
                        if (k == j || k >= placed) continue;
                        if (clash_pair(m, mols[k], bx.L, rmin2)) return true;
                    }
                }
        return false;
    }
    for (int k = 0; k < placed; k++) {
        if (k == j) continue;
        if (clash_pair(m, mols[k], bx.L, rmin2)) return true;
    }
    return false;
}

void cell_move(Box &bx, int j, const double o_new[3]) {
    if (bx.nc < 3) return;
    int cnew = bx.cell_index(o_new);
    int cold = bx.cell_of[j];
    if (cnew == cold) return;
    auto &v = bx.members[cold];
    for (size_t i = 0; i < v.size(); i++)
        if (v[i] == j) { v[i] = v.back(); v.pop_back(); break; }
    bx.members[cnew].push_back(j);
    bx.cell_of[j] = cnew;
}

void emit(const std::vector<Mol> &mols, float *xyz) {
    for (size_t j = 0; j < mols.size(); j++) {
        double R[3][3];
        rotmat(mols[j].q, R);
        for (int s = 0; s < 4; s++)
            for (int a = 0; a < 3; a++)
                xyz[(j * 4 + s) * 3 + a] =
                    (float)(mols[j].o[a] + R[a][0] * BODY[s][0] + R[a][1] * BODY[s][1] + R[a][2] * BODY[s][2]);
    }
}

}  // namespace

extern "C" int cir_synth_default(cir_synth *s, int nmol) {
    if (!s) return cir_fail(CIR_ERR_ARG, "cir_synth_default: null pointer");
    s->nmol = nmol;
    s->seed = 1;
    s->box_nm = 0;
    s->frame_dt = 0.010;
    s->sigma_trans = 0.003;
    s->sigma_rot_deg = 3.0;
    s->jitter = 0.02;
    s->min_contact = 0.15;
    s->max_tries = 8;
    return CIR_OK;
}

extern "C" int cir_synth_trajectory(const cir_synth *s, int nframes, float *xyz, float *box,
                                    long long *n_rejected) {
    if (!s || !xyz || nframes < 1 || s->nmol < 2 || s->nmol > 1000000)
        return cir_fail(CIR_ERR_ARG, "cir_synth_trajectory: bad argument");
    const int nmol = s->nmol;
    const double L = s->box_nm > 0 ? s->box_nm : 1.2417 * cube_root((double)nmol / 64.0);
    const double rmin2 = s->min_contact * s->min_contact;
    const double rot_sigma = s->sigma_rot_deg * (3.14159265358979323846 / 180.0);
    const int tries = s->max_tries > 0 ? s->max_tries : 1;

    Box bx;
    bx.L = L;
    // an O..O distance below min_contact + 2 r_OH is needed for any O/H contact
    const double rc = s->min_contact + 2 * R_OH;
    bx.nc = (int)(L / rc);
    if (bx.nc >= 3) {
        bx.members.assign((size_t)bx.nc * bx.nc * bx.nc, {});
        bx.cell_of.assign(nmol, 0);
    }

    std::vector<Mol> mols(nmol);
    long long rejected = 0;
    int c = 1;
    while ((long long)c * c * c < nmol) c++;
    const double a = L / c;
    for (int j = 0; j < nmol; j++) {
        const int ix = j % c, iy = (j / c) % c, iz = j / (c * c);
        bool ok = false;
        for (int att = 0; att < 100000 && !ok; att++) {
            Stream st(s->seed, 0, (uint64_t)j, (uint64_t)att);
            Mol m;
            m.o[0] = (ix + 0.5) * a + s->jitter * (2 * st.uniform() - 1);
            m.o[1] = (iy + 0.5) * a + s->jitter * (2 * st.uniform() - 1);
            m.o[2] = (iz + 0.5) * a + s->jitter * (2 * st.uniform() - 1);
            for (int d = 0; d < 3; d++) m.o[d] = wrap(m.o[d], L);
            st.quat(m.q);
            place(m);
            if (!clashes(m, j, mols, j, bx, rmin2)) {
                mols[j] = m;
                ok = true;
            } else {
                rejected++;
            }
        }
        if (!ok) return cir_fail(CIR_ERR_ARG, "cir_synth_trajectory: cannot place molecule %d without contacts", j);
        if (bx.nc >= 3) {
            int cc = bx.cell_index(mols[j].o);
            bx.cell_of[j] = cc;
            bx.members[cc].push_back(j);
        }
    }
    const size_t fstride = (size_t)nmol * 4 * 3;
    emit(mols, xyz);
    for (int f = 1; f < nframes; f++) {
        for (int j = 0; j < nmol; j++) {
            for (int att = 0; att < tries; att++) {
                Stream st(s->seed, (uint64_t)f, (uint64_t)j, (uint64_t)att);
                Mol m = mols[j];
                for (int d = 0; d < 3; d++) m.o[d] = wrap(m.o[d] + s->sigma_trans * st.gauss(), L);
                double u[3];
                st.unit3(u);
                const double half = 0.5 * rot_sigma * st.gauss();
                double dq[4] = {1.0, u[0] * half, u[1] * half, u[2] * half};
                qnorm(dq);
                double qn[4];
                qmul(dq, mols[j].q, qn);
                qnorm(qn);
                memcpy(m.q, qn, sizeof qn);
                place(m);
                if (!clashes(m, j, mols, nmol, bx, rmin2)) {
                    cell_move(bx, j, m.o);
                    mols[j] = m;
                    break;
                }
                rejected++;
            }
        }
        emit(mols, xyz + (size_t)f * fstride);
    }
    if (box) box[0] = box[1] = box[2] = (float)L;
    if (n_rejected) *n_rejected = rejected;
    return CIR_OK;
}
