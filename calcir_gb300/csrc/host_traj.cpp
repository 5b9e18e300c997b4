// Raw trajectory files ("CIRTRJ01"): the random-access frame source of the drop-in
// executable for user-supplied positions.  Layout (little endian):
//   char magic[8] = "CIRTRJ01"; int32 natoms; int32 nframes; float32 frame_dt; int32 0;
//   per frame: float32 time; float32 box[3]; float32 xyz[natoms][3]   (nm, ps)
// cir_traj_info / cir_traj_read also read GROMACS .xtc files (detected by their magic
// number, host_xtc.cpp); together they stand in for read_xtc_natoms / read_xtc_n_frames /
// xdr_seek / read_xtc (calcIR.cu:212-223, 341-352, 376-395).
#include "cir_internal.h"

#include <cstdio>
#include <cstring>

static const char MAGIC[8] = {'C', 'I', 'R', 'T', 'R', 'J', '0', '1'};

extern "C" int cir_traj_write(const char *path, int natoms, int nframes, float frame_dt,
                              const float *times, const float *boxes, const float *xyz) {
    if (!path || natoms < 1 || nframes < 1 || !boxes || !xyz)
        return cir_fail(CIR_ERR_ARG, "cir_traj_write: bad argument");
    FILE *f = fopen(path, "wb");
    if (!f) return cir_fail(CIR_ERR_IO, "cannot open %s for writing", path);
    int32_t hdr[4] = {natoms, nframes, 0, 0};
    memcpy(&hdr[2], &frame_dt, 4);
    bool ok = fwrite(MAGIC, 1, 8, f) == 8 && fwrite(hdr, 4, 4, f) == 4;
    for (int i = 0; ok && i < nframes; i++) {
        float t = times ? times[i] : i * frame_dt;
        ok = fwrite(&t, 4, 1, f) == 1 && fwrite(boxes + 3 * (size_t)i, 4, 3, f) == 3 &&
             fwrite(xyz + (size_t)i * natoms * 3, 4, (size_t)natoms * 3, f) == (size_t)natoms * 3;
    }
    if (fclose(f) != 0) ok = false;
    return ok ? CIR_OK : cir_fail(CIR_ERR_IO, "write to %s failed", path);
}

static FILE *open_checked(const char *path, int32_t hdr[4]) {
    FILE *f = fopen(path, "rb");
    if (!f) return nullptr;
    char m[8];
    if (fread(m, 1, 8, f) != 8 || memcmp(m, MAGIC, 8) != 0 || fread(hdr, 4, 4, f) != 4) {
        fclose(f);
        return nullptr;
    }
    return f;
}

extern "C" int cir_traj_info(const char *path, int *natoms, int *nframes, float *frame_dt) {
    if (path && cir_is_xtc(path)) return cir_xtc_info(path, natoms, nframes, frame_dt);
    int32_t hdr[4];
    FILE *f = path ? open_checked(path, hdr) : nullptr;
    if (!f) return cir_fail(CIR_ERR_IO, "WARNING: The file %s could not be opened as a CIRTRJ01 trajectory.", path ? path : "(null)");
    fclose(f);
    if (natoms) *natoms = hdr[0];
    if (nframes) *nframes = hdr[1];
    if (frame_dt) memcpy(frame_dt, &hdr[2], 4);
    return CIR_OK;
}

extern "C" int cir_traj_read(const char *path, int first, int count, float *xyz, float *boxes, float *times) {
    if (path && cir_is_xtc(path)) return cir_xtc_read(path, first, count, xyz, boxes, times);
    int32_t hdr[4];
    FILE *f = path ? open_checked(path, hdr) : nullptr;
    if (!f) return cir_fail(CIR_ERR_IO, "cannot open %s as a CIRTRJ01 trajectory", path ? path : "(null)");
    const int natoms = hdr[0], nframes = hdr[1];
    if (first < 0 || count < 0 || first + count > nframes) {
        fclose(f);
        return cir_fail(CIR_ERR_ARG, "frames [%d, %d) outside the %d frames of %s", first, first + count, nframes, path);
    }
    const long long fbytes = 16 + 12LL * natoms;
    bool ok = fseek(f, 24 + fbytes * first, SEEK_SET) == 0;
    for (int i = 0; ok && i < count; i++) {
        float t, b[3];
        ok = fread(&t, 4, 1, f) == 1 && fread(b, 4, 3, f) == 3;
        if (!ok) break;
        if (times) times[i] = t;
        if (boxes) memcpy(boxes + 3 * (size_t)i, b, 12);
        if (xyz) ok = fread(xyz + (size_t)i * natoms * 3, 4, (size_t)natoms * 3, f) == (size_t)natoms * 3;
        else ok = fseek(f, 12LL * natoms, SEEK_CUR) == 0;
    }
    fclose(f);
    return ok ? CIR_OK : cir_fail(CIR_ERR_IO, "short read from %s", path);
}
