// Field projection, spectroscopic maps and the exciton Hamiltonian of a batch of frames.
//
// k_chromophore: one thread per chromophore.  The field at H_c sums the H1/H2 (+0.52)
// and M (-1.04) charges of every other molecule whose O lies within 0.7831 nm of H_c
// (minimum image), projected on the OH unit vector (get_eproj_GPU, calcIR.cu:1020-1168).
// Molecules are staged through shared memory in tiles.  The same thread then evaluates
// the maps and writes the per-chromophore table, the dipole and the polarisability
// (calcIR.cu:1256-1304).
//
// k_hmatrix: one 32x32 tile of H per block (get_kappa_GPU, calcIR.cu:1306-1402).  Every
// pair is evaluated with its lower index first, so H is exactly symmetric and both
// triangles are written with coalesced stores.
#include "cir_device.cuh"

namespace {

constexpr int CHROM_THREADS = 128;
constexpr int MOL_TILE = 128;

__global__ void __launch_bounds__(CHROM_THREADS) k_chromophore(BuildArgs a) {
    __shared__ float sm_mol[MOL_TILE][10];   // O(3), H1(3), H2(3) ... M stored separately
    __shared__ float sm_m[MOL_TILE][3];
    __shared__ int sm_hasm;
    const int f = blockIdx.y;
    const int c = blockIdx.x * CHROM_THREADS + threadIdx.x;
    const float *x = a.xyz + (size_t)f * a.natoms * 3;
    const float bx = a.box[3 * f], by = a.box[3 * f + 1], bz = a.box[3 * f + 2];
    const bool active = c < a.n;

    int n = 0;
    float hx = 0, hy = 0, hz = 0, ox = 0, oy = 0, oz = 0, ux = 0, uy = 0, uz = 1;
    if (active) {
        n = c / a.nchrom_mol;
        const int hatom = n * a.natom_mol + 1 + (c % 2);   // chrom%2 selects HW1/HW2 (calcIR.cu:1061-1072)
        hx = x[3 * hatom]; hy = x[3 * hatom + 1]; hz = x[3 * hatom + 2];
        const int oatom = n * a.natom_mol;
        ox = x[3 * oatom]; oy = x[3 * oatom + 1]; oz = x[3 * oatom + 2];
        ux = cir_mi(hx - ox, bx); uy = cir_mi(hy - oy, by); uz = cir_mi(hz - oz, bz);
        const float r = sqrtf(ux * ux + uy * uy + uz * uz);
        ux /= r; uy /= r; uz /= r;
    }
    if (threadIdx.x == 0) sm_hasm = a.natom_mol >= 4;
    float ex = 0, ey = 0, ez = 0;
    for (int t0 = 0; t0 < a.nmol; t0 += MOL_TILE) {
        __syncthreads();
        const int m = t0 + threadIdx.x;
        if (threadIdx.x < MOL_TILE && m < a.nmol) {
            const float *mo = x + (size_t)m * a.natom_mol * 3;
            #pragma unroll
            for (int q = 0; q < 9; q++) sm_mol[threadIdx.x][q] = mo[q];
            if (a.natom_mol >= 4) {
                float mx = mo[9], my = mo[10], mz = mo[11];
                if (a.imodel != 0) {   // move M to the TIP4P distance (calcIR.cu:1131-1146)
                    const float dx = cir_mi(mx - mo[0], bx), dy = cir_mi(my - mo[1], by), dz = cir_mi(mz - mo[2], bz);
                    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
                    mx = mo[0] + CIR_OM_TIP4P * dx / r;
                    my = mo[1] + CIR_OM_TIP4P * dy / r;
                    mz = mo[2] + CIR_OM_TIP4P * dz / r;
                }
                sm_m[threadIdx.x][0] = mx; sm_m[threadIdx.x][1] = my; sm_m[threadIdx.x][2] = mz;
            }
        }
        __syncthreads();
        if (!active) continue;
        const int tn = min(MOL_TILE, a.nmol - t0);
        for (int j = 0; j < tn; j++) {
            if (t0 + j == n) continue;
            const float *mo = sm_mol[j];
            const float dx = cir_mi(mo[0] - hx, bx), dy = cir_mi(mo[1] - hy, by), dz = cir_mi(mo[2] - hz, bz);
            if (cir_mag3(dx, dy, dz) > CIR_CUTOFF) continue;   // calcIR.cu:1106-1113
            #pragma unroll
            for (int s = 0; s < 3; s++) {
                float sx, sy, sz, q;
                if (s < 2) { sx = mo[3 + 3 * s]; sy = mo[4 + 3 * s]; sz = mo[5 + 3 * s]; q = CIR_QH; }
                else {
                    if (!sm_hasm) break;
                    sx = sm_m[j][0]; sy = sm_m[j][1]; sz = sm_m[j][2]; q = -CIR_QM;
                }
                const float qx = cir_mi(hx - sx, bx) * CIR_BOHR_NM;
                const float qy = cir_mi(hy - sy, by) * CIR_BOHR_NM;
                const float qz = cir_mi(hz - sz, bz) * CIR_BOHR_NM;
                const float rr = sqrtf(qx * qx + qy * qy + qz * qz);
                const float s3 = q / (rr * rr * rr);
                ex += s3 * qx; ey += s3 * qy; ez += s3 * qz;
            }
        }
    }
    if (!active) return;
    const float E = ex * ux + ey * uy + ez * uz;
    const CirMaps &mp = a.maps;
    const float w = mp.w[0] + mp.w[1] * E + mp.w[2] * E * E;
    const float xm = mp.x[0] + mp.x[1] * w;
    const float pm = mp.p[0] + mp.p[1] * w;
    const float mup = mp.mup[0] + mp.mup[1] * E + mp.mup[2] * E * E;
    // transition dipole position, each coordinate wrapped by minImage (calcIR.cu:1288-1291)
    const float tx = cir_mi(ox + CIR_TDM_OFFSET * ux, bx);
    const float ty = cir_mi(oy + CIR_TDM_OFFSET * uy, by);
    const float tz = cir_mi(oz + CIR_TDM_OFFSET * uz, bz);
    float *ct = a.ct + (size_t)f * CT_NROW * a.ld;
    ct[CT_E * a.ld + c] = E;
    ct[CT_W * a.ld + c] = w;
    ct[CT_X * a.ld + c] = xm;
    ct[CT_P * a.ld + c] = pm;
    ct[CT_MUP * a.ld + c] = mup;
    ct[CT_UX * a.ld + c] = ux; ct[CT_UY * a.ld + c] = uy; ct[CT_UZ * a.ld + c] = uz;
    ct[CT_TX * a.ld + c] = tx; ct[CT_TY * a.ld + c] = ty; ct[CT_TZ * a.ld + c] = tz;
    if (a.eproj) a.eproj[(size_t)f * a.n + c] = E;
    if (a.dip) {   // calcIR.cu:1294-1296
        float *d = a.dip + (size_t)f * a.dip_fstride;
        const float s = mup * xm;
        d[c] = ux * s; d[a.ldv + c] = uy * s; d[2 * a.ldv + c] = uz * s;
    }
    if (a.pol) {   // calcIR.cu:1299-1304
        float *p = a.pol + (size_t)f * a.pol_fstride;
        p[c] = (4.6f * ux * ux + 1.0f) * xm;
        p[a.ldv + c] = (4.6f * uy * uy + 1.0f) * xm;
        p[2 * a.ldv + c] = (4.6f * uz * uz + 1.0f) * xm;
        p[3 * a.ldv + c] = 4.6f * ux * uy * xm;
        p[4 * a.ldv + c] = 4.6f * uy * uz * xm;
        p[5 * a.ldv + c] = 4.6f * uz * ux * xm;
    }
}

struct Chrom {
    float E, w, x, p, mup, ux, uy, uz, tx, ty, tz;
    int mol;
};

__device__ __forceinline__ float pair_coupling(const Chrom &lo, const Chrom &hi, float bx, float by, float bz,
                                               const CirMaps &mp, int ispecies) {
    if (ispecies == 1 || ispecies == 2) return 0.f;       // HOD: no coupling (calcIR.cu:1334, 1348)
    if (lo.mol == hi.mol)                                   // intramolecular map (calcIR.cu:1339)
        return (mp.wi[0] + mp.wi[1] * (lo.E + hi.E)) * lo.x * hi.x + mp.wi[2] * lo.p * hi.p;
    // transition dipole coupling (calcIR.cu:1352-1399)
    float dx = cir_mi(lo.tx - hi.tx, bx), dy = cir_mi(lo.ty - hi.ty, by), dz = cir_mi(lo.tz - hi.tz, bz);
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    dx /= r; dy /= r; dz /= r;
    r *= CIR_BOHR_NM;
    const float uu = lo.ux * hi.ux + lo.uy * hi.uy + lo.uz * hi.uz;
    const float un = lo.ux * dx + lo.uy * dy + lo.uz * dz;
    const float vn = hi.ux * dx + hi.uy * dy + hi.uz * dz;
    return (uu - 3.0f * un * vn) / (r * r * r) * lo.x * hi.x * lo.mup * hi.mup * CIR_CM_HARTREE;
}

constexpr int HT = 32;   // tile edge
__global__ void __launch_bounds__(HT * 8) k_hmatrix(BuildArgs a) {
    // H is symmetric and each coupling is evaluated in canonical order (the lower index
    // first), so a tile above the diagonal is computed once and written twice: directly and,
    // through shared memory, transposed into its mirror tile; tiles below the diagonal return
    if (blockIdx.y > blockIdx.x) return;
    __shared__ Chrom rows[HT], cols[HT];
    __shared__ float tile[HT][HT + 1];
    const int f = blockIdx.z;
    const int r0 = blockIdx.y * HT, c0 = blockIdx.x * HT;
    const bool mirror = blockIdx.y < blockIdx.x;
    const float *ct = a.ct + (size_t)f * CT_NROW * a.ld;
    const int tid = threadIdx.y * HT + threadIdx.x;
    if (tid < 2 * HT) {
        const int loc = tid % HT;
        const int idx = (tid < HT ? r0 : c0) + loc;
        Chrom ch = {};
        if (idx < a.n) {
            ch.E = ct[CT_E * a.ld + idx]; ch.w = ct[CT_W * a.ld + idx]; ch.x = ct[CT_X * a.ld + idx];
            ch.p = ct[CT_P * a.ld + idx]; ch.mup = ct[CT_MUP * a.ld + idx];
            ch.ux = ct[CT_UX * a.ld + idx]; ch.uy = ct[CT_UY * a.ld + idx]; ch.uz = ct[CT_UZ * a.ld + idx];
            ch.tx = ct[CT_TX * a.ld + idx]; ch.ty = ct[CT_TY * a.ld + idx]; ch.tz = ct[CT_TZ * a.ld + idx];
            ch.mol = idx / a.nchrom_mol;
        }
        (tid < HT ? rows : cols)[loc] = ch;
    }
    __syncthreads();
    const float bx = a.box[3 * f], by = a.box[3 * f + 1], bz = a.box[3 * f + 2];
    const int c = c0 + threadIdx.x;
    float *H = a.H + (size_t)f * a.n * a.ldh;
    #pragma unroll
    for (int i = 0; i < HT / 8; i++) {
        const int rl = threadIdx.y + 8 * i;
        const int r = r0 + rl;
        if (r >= a.n || c >= a.n) continue;
        float h;
        if (r == c) h = rows[rl].w - a.avef;               // calcIR.cu:1322-1328
        else if (r < c) h = pair_coupling(rows[rl], cols[threadIdx.x], bx, by, bz, a.maps, a.ispecies);
        else h = pair_coupling(cols[threadIdx.x], rows[rl], bx, by, bz, a.maps, a.ispecies);
        H[(size_t)r * a.ldh + c] = h;
        tile[rl][threadIdx.x] = h;
    }
    if (!mirror) return;
    __syncthreads();
    // the mirror tile: H[c0 + j][r0 + l] = H[r0 + l][c0 + j], written along r0 + l
    const int rm = r0 + threadIdx.x;
    #pragma unroll
    for (int i = 0; i < HT / 8; i++) {
        const int jl = threadIdx.y + 8 * i, cm = c0 + jl;
        if (cm < a.n && rm < a.n) H[(size_t)cm * a.ldh + rm] = tile[threadIdx.x][jl];
    }
}

}  // namespace

cudaError_t cir_launch_build(const BuildArgs &a, int nframes, cudaStream_t s, int *launches) {
    dim3 g1((a.n + CHROM_THREADS - 1) / CHROM_THREADS, nframes);
    k_chromophore<<<g1, CHROM_THREADS, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 g2((a.n + HT - 1) / HT, (a.n + HT - 1) / HT, nframes);
    k_hmatrix<<<g2, dim3(HT, 8), 0, s>>>(a);
    if (launches) *launches += 2;
    return cudaGetLastError();
}
