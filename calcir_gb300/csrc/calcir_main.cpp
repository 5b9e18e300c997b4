// calcir: drop-in for `calcIR.exe input.inp`.  Reads the same input keys, builds the
// frames (a CIRTRJ01 trajectory file or the seeded synthetic generator, selected with
// `xtcf synthetic`), runs the whole job on the GPU through the C ABI and writes the 13
// output files with the reference's names and formats (calcIR.cu:9-1012).
#include "calcir.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <vector>

static int die(const char *what) {
    printf("%s\n", what);
    return EXIT_FAILURE;
}

int main(int argc, char *argv[]) {
    if (argc != 2) {   // calcIR.cu:14-18
        printf("Usage:\n"
               "\tInclude as the first argument the name of an input file. No other arguments are allowed.\n");
        return EXIT_FAILURE;
    }
    const time_t start = time(NULL);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess)
        printf("\nGPU INFO:\n\tDevice name: %s\n\tMemory: %g gb\n", prop.name, prop.totalGlobalMem / (1.E9));
    printf("\n>>> Setting default parameters\n");
    cir_params p;
    cir_params_default(&p);
    p.verbose = 1;
    if (cir_params_parse_file(argv[1], &p) != CIR_OK) return die(cir_last_error());
    printf("\tSetting xtc file %s\n", p.xtcf);
    printf("\tSetting default file name to %s\n", p.outf);
    printf("\tSetting model to %s\n", p.model);
    printf("\tSetting the number of tcf points to %d\n", p.ntcfpoints);
    printf("\tSetting nsamples to %d\n", p.nsamples);
    printf("\tSetting sampleEvery to %f (ps)\n", p.sampleEvery);
    printf("\tSetting omegaStep to %d\n", p.omegaStep);
    printf("\tSetting natom_mol to %d\n", p.natom_mol);
    printf("\tSetting nchrom_mol to %d\n", p.nchrom_mol);
    printf("\tSetting nzeros to %d\n", p.nzeros);
    printf("\tSetting map to %d\n", p.map);
    printf("\tSetting species to %s\n", p.species);
    printf("\tSetting omegaStart to %f\n", p.omegaStart);
    printf("\tSetting omegaStop to %f\n", p.omegaStop);
    printf("\tSetting dt to %f\n", p.dt);
    printf("\tSetting t1 to %f (ps)\n", p.t1);
    printf("\tSetting avef to %f\n", p.avef);
    printf("\tSetting equilibration time to %f (ps)\n", p.beginTime);
    if (cir_params_finalize(&p) != CIR_OK) return die(cir_last_error());

    // frame of every (sample, step) (calcIR.cu:378-379)
    const bool synthetic = strcmp(p.xtcf, "synthetic") == 0;
    int natoms = 0, nframes_file = 0;
    float frame_dt = 0;
    if (synthetic) {
        if (p.natom_mol != 4) return die("ERROR: the synthetic source writes 4 atoms per molecule (natom_mol 4)");
        natoms = 4 * p.synth_nmol;
        frame_dt = p.synth_frame_dt;
    } else {
        if (cir_traj_info(p.xtcf, &natoms, &nframes_file, &frame_dt) != CIR_OK) return die(cir_last_error());
    }
    const int nmol = natoms / p.natom_mol;
    printf(">>> Will read the trajectory from: %s.\n", p.xtcf);
    printf(">>> Found %d atoms and %d molecules.\n", natoms, nmol);
    printf(">>> Found %d chromophores.\n", nmol * p.nchrom_mol);
    printf(">>> Frame time offset is: %f (ps)\n", frame_dt);
    const int S = p.nsamples, K = p.ntcfpoints;
    std::vector<int> step_frame((size_t)S * K);
    int fmax = 0;
    for (int s = 0; s < S; s++)
        for (int k = 0; k < K; k++) {
            int f;
            cir_frame_index(&p, frame_dt, s, k, &f);
            if (f < 0) return die("WARNING:: a requested frame lies before the start of the trajectory.");
            step_frame[(size_t)s * K + k] = f;
            if (f > fmax) fmax = f;
        }
    // distinct frames, in increasing order
    std::map<int, int> slot;
    for (int f : step_frame) slot[f] = 0;
    std::vector<int> frames;
    for (auto &kv : slot) { kv.second = (int)frames.size(); frames.push_back(kv.first); }
    const int nfr = (int)frames.size();
    std::vector<float> xyz((size_t)nfr * natoms * 3), box((size_t)nfr * 3);
    if (synthetic) {
        cir_synth sy;
        cir_synth_default(&sy, p.synth_nmol);
        sy.seed = (uint64_t)p.synth_seed;
        sy.frame_dt = p.synth_frame_dt;
        sy.sigma_trans = p.synth_sigma_trans;
        sy.sigma_rot_deg = p.synth_sigma_rot;
        std::vector<float> all((size_t)(fmax + 1) * natoms * 3);
        float b3[3];
        if (cir_synth_trajectory(&sy, fmax + 1, all.data(), b3, nullptr) != CIR_OK) return die(cir_last_error());
        for (int i = 0; i < nfr; i++) {
            memcpy(&xyz[(size_t)i * natoms * 3], &all[(size_t)frames[i] * natoms * 3], (size_t)natoms * 12);
            memcpy(&box[3 * (size_t)i], b3, 12);
        }
    } else {
        if (fmax >= nframes_file) return die("WARNING:: the trajectory is shorter than the requested samples.");
        printf(">>> Now indexing the xtc file to allow random access.\n");
        for (int i = 0; i < nfr; i++) {
            float t;
            if (cir_traj_read(p.xtcf, frames[i], 1, &xyz[(size_t)i * natoms * 3], &box[3 * (size_t)i], &t) != CIR_OK)
                return die(cir_last_error());
            // the frame time check of calcIR.cu:391-395, for the first step that uses it
            for (int s = 0; s < S; s++)
                for (int k = 0; k < K; k++)
                    if (step_frame[(size_t)s * K + k] == frames[i]) {
                        const float desired = s * p.sampleEvery + p.beginTime + p.dt * k;
                        if (fabsf(desired - t) > frame_dt * 1E-1f) {
                            printf("\nWARNING:: could not find the desired frame at time %f (ps).\n", desired);
                            printf("I am instead at gmxtime: %f.\nIs something wrong with the trajectory?", t);
                            return EXIT_FAILURE;
                        }
                        s = S;
                        break;
                    }
        }
    }
    for (auto &f : step_frame) f = slot[f];

    printf("\n>>> Now calculating the absorption spectrum\n");
    printf("----------------------------------------------------------\n");
    cir_ctx *ctx = nullptr;
    if (cir_create(&p, natoms, &ctx) != CIR_OK) return die(cir_last_error());
    int ntcf, nomega, nls;
    cir_result_sizes(&p, &ntcf, &nomega, &nls);
    std::vector<double> tir(2 * ntcf), tvv(2 * ntcf), tvh(2 * ntcf);
    std::vector<float> om(nomega), sw(nomega), pw(nomega), rw(nomega), rmw(nomega);
    std::vector<float> lo(nls), li(nls), lv(nls), lh(nls);
    cir_result r;
    memset(&r, 0, sizeof r);
    r.tcf_ir = tir.data(); r.tcf_vv = tvv.data(); r.tcf_vh = tvh.data();
    r.omega = om.data(); r.sw = sw.data(); r.pw = pw.data(); r.rw = rw.data(); r.rmw = rmw.data();
    r.ls_omega = lo.data(); r.ls_ir = li.data(); r.ls_vv = lv.data(); r.ls_vh = lh.data();
    if (cir_run(ctx, nfr, xyz.data(), box.data(), step_frame.data(), &r) != CIR_OK) {
        printf("ERROR: %s\n", cir_last_error());
        cir_destroy(ctx);
        return EXIT_FAILURE;
    }
    cir_destroy(ctx);
    if (r.bins_out_of_range)
        printf("WARNING: %lld eigenvalues fell outside [omegaStart, omegaStop] and were not binned.\n",
               r.bins_out_of_range);
    printf("\n\n----------------------------------------------------------\n");
    printf("Finishing up...\n");
    if (cir_write_outputs(&p, &r) != CIR_OK) return die(cir_last_error());
    printf(">>> %.1f frame-steps/s on the device\n", r.frame_steps_per_s);
    printf("\n>>> Done with the calculation in %f seconds.\n", difftime(time(NULL), start));
    return 0;
}
