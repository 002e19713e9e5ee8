// emoopic_main.cpp - the EMOOPIC driver on the GPU library: same command line
// (one input file), same initialisation order and time loop as the reference
// driver (src/main.cpp:45-336), through the class API of emoopic.hpp.
//
//   emoopic_gpu <input.txt> [--mixed] [--dt DT] [--multigrid] [--corrected]
//
// --multigrid solves the "poisson" field start by multigrid instead of the
// reference's Jacobi (EMOO_POISSON_MULTIGRID); --corrected selects the
// corrected-physics policy (EMOO_POLICY_CORRECTED).
//
// Writes history.dat next to the input file like the reference, and the field
// time series at the reference's cadence (t = 0, every nstep_fields steps, the
// last step) into output.fields/ there: the reference's HDF5 datasets as raw
// files (emoo_write_fields; HDF5 is not available). With nstep_restart > 0 it
// writes restart.emoo there every nstep_restart steps; with restart = 1 in the
// input it continues from that file when present. Particle tracks of the
// reference are not part of this program.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <string>

#include "emoopic.hpp"

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <input.txt> [--mixed] [--dt DT] [--multigrid] [--corrected]\n", argv[0]);
        return 1;
    }
    emoo_opts &opt = emoopic::Options::get().o;
    for (int a = 2; a < argc; a++) {
        if (!strcmp(argv[a], "--mixed")) opt.precision = EMOO_MIXED;
        else if (!strcmp(argv[a], "--dt") && a + 1 < argc) opt.dt = atof(argv[++a]);
        else if (!strcmp(argv[a], "--multigrid")) opt.poisson_solver = EMOO_POISSON_MULTIGRID;
        else if (!strcmp(argv[a], "--corrected")) opt.policy = EMOO_POLICY_CORRECTED;
        else {
            fprintf(stderr, "unknown option %s\n", argv[a]);
            return 1;
        }
    }
    clock_t begin = clock();
    try {
        Input input;
        if (input.readinfo(argv[1])) return 1;
        if (input.ProcessInfo()) {
            fprintf(stderr, "Input is inconsistent\n");
            return 1;
        }
        Input_Info_t *info = input.getinfo();
        Domain domain(info);
        Particle_Handler part_handler;
        Pusher *pusher = info->relativity ? (Pusher *)new Relativistic_Boris() : (Pusher *)new Boris();
        part_handler.setPusher(pusher);
        BC_Particle **bc = Part_BC_Factory::getInstance().constructConditions(&domain, info);
        part_handler.setParticleBoundaries(bc);
        bool poisson = info->restart == 0 && strcmp(info->fields_init, "poisson") == 0;
        Grid *grids = poisson ? new Poisson_Solver(&domain, info) : new Grid(&domain, info);
        Field_BC_Factory::getInstance().Construct(&domain, grids, info);
        part_handler.attach(grids);
        part_handler.Load(info, &domain);
        if (poisson) {
            part_handler.depositRhoJ(grids, true, &domain, info);
            grids->executeBC(EMOO_SEND_JRHO);
        }
        grids->InitializeFields(info);
        std::string inputname = argv[1];
        std::string dir = inputname.substr(0, inputname.find_last_of('/') + 1);
        OutputBoxQuantities box((dir + "history.dat").c_str(), grids, &part_handler, info);
        emoo_handle *h = grids->handle();
        double t = info->t0, dt = 0.0;
        emoo_time(h, nullptr, &dt);
        const std::string fields_dir = dir + "output.fields", restart = dir + "restart.emoo";
        int t0 = 0;
        if (info->restart) {
            FILE *rf = fopen(restart.c_str(), "rb");
            if (rf) {
                fclose(rf);
                emoopic::check(emoo_read_restart(h, restart.c_str()), "emoo_read_restart");
                emoo_time(h, &t, nullptr);
                t0 = (int)llround((t - info->t0) / dt);
                printf("Continuing from %s at step %d\n", restart.c_str(), t0);
            }
        }
        const int nstep_fields = info->nstep_fields > 0 ? info->nstep_fields : 1;
        if (info->which_fields >= 0 && t0 == 0)
            emoopic::check(emoo_write_fields(h, fields_dir.c_str(), info->which_fields), "emoo_write_fields");
        printf("Advancing %d time steps with dt = %f\n", info->nt, dt);
        int64_t cross[6];
        for (int ti = t0; ti < info->nt; ti++) {
            box.output(t, ti);
            // sort (every nstep_sort) + fused push / boundaries / deposit +
            // fold + Yee update + E/B boundaries, src/main.cpp:225-272
            emoopic::check(emoo_step(h, 1, cross), "emoo_step");
            t += dt;
            // output, src/main.cpp:277-283
            if ((ti + 1) % nstep_fields == 0 && info->which_fields >= 0)
                emoopic::check(emoo_write_fields(h, fields_dir.c_str(), info->which_fields), "emoo_write_fields");
            if (info->nstep_restart > 0 && (ti + 1) % info->nstep_restart == 0)
                emoopic::check(emoo_write_restart(h, restart.c_str()), "emoo_write_restart");
        }
        printf("***Timestep loop complete***\n");
        // final output, src/main.cpp:295-300
        if (info->nt % nstep_fields != 0 && info->which_fields >= 0)
            emoopic::check(emoo_write_fields(h, fields_dir.c_str(), info->which_fields), "emoo_write_fields");
        delete grids;
        for (int i = 0; i < 6; i++) delete bc[i];
        delete[] bc;
        delete pusher;
    } catch (const std::exception &e) {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    printf("Program completed successfully!\nElapsed: %f seconds\n", (double)(clock() - begin) / CLOCKS_PER_SEC);
    return 0;
}
