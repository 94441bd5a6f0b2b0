// e2d_solve -- command-line drop-in for the reference program (gpu_fvm.cu:27-68).
//
// Reads the mesh (default "2822-3k.dat", as gpu_init.cu:10) and input.dat
// (gpu_init.cu:35) from the working directory, prints "step,resid" per
// iteration (gpu_solver.cu:2433), and writes unresult.plt, unresidual.plt and
// unairfoilpress.plt (gpu_fvm.cu:133-195) with the converged field.
//
//   e2d_solve [mesh.dat [input.dat]] [--fp32] [--file-order] [--out DIR]
//             [--global-dt] [--far-field-fix]
// --global-dt advances every cell with the smallest local step; --far-field-fix
// makes the far-field supersonic test use the non-dimensional sound speed.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/time.h>
#include <vector>

#include "euler2d.h"

static int fail(const char *what) {
    std::printf("%s: %s\n", what, e2d_last_error());
    return 1;
}

int main(int argc, char **argv) {
    std::string mesh_path = "2822-3k.dat", input_path = "input.dat", out = ".";
    int precision = E2D_FP64, ordering = E2D_ORDER_MORTON, npos = 0, global_dt = 0, far_fix = 0;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--fp32")) precision = E2D_FP32;
        else if (!std::strcmp(argv[i], "--file-order")) ordering = E2D_ORDER_FILE;
        else if (!std::strcmp(argv[i], "--out") && i + 1 < argc) out = argv[++i];
        else if (!std::strcmp(argv[i], "--global-dt")) global_dt = 1;
        else if (!std::strcmp(argv[i], "--far-field-fix")) far_fix = 1;
        else if (argv[i][0] == '-') {
            std::printf("usage: e2d_solve [mesh.dat [input.dat]] [--fp32] [--file-order] [--out DIR] "
                        "[--global-dt] [--far-field-fix]\n");
            return 2;
        } else if (npos++ == 0) mesh_path = argv[i];
        else input_path = argv[i];
    }
    e2d_mesh *m = nullptr;
    if (e2d_mesh_read(mesh_path.c_str(), &m)) {
        std::printf("\nCannot open the mesh data file!\n");
        return 1;
    }
    e2d_params p;
    e2d_params_default(&p);
    if (e2d_input_read(input_path.c_str(), &p)) {
        std::printf("\nCannot open input file!\n");
        return 1;
    }
    std::printf("inputData finished!\n");
    e2d_mesh_info info;
    if (e2d_mesh_info_get(m, p.wall_box, &info)) return fail("mesh");
    std::printf("Mesh data Computing's finished!!\n");
    p.precision = precision;
    p.ordering = ordering;
    p.global_dt = global_dt;
    p.far_field_fix = far_fix;
    p.verbose = 1;
    e2d_solver *s = nullptr;
    if (e2d_solver_create(m, &p, &s)) return fail("solver");
    struct timeval t0, t1;
    gettimeofday(&t0, nullptr);
    std::vector<double> hist(p.maxstep > 0 ? p.maxstep : 1);
    int32_t n = 0;
    int rc = e2d_solve(s, p.maxstep, p.epsl, hist.data(), &n);
    gettimeofday(&t1, nullptr);
    std::printf("total time: %g\n", (double)(t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec));
    if (rc) std::printf("solver stopped: %s\n", e2d_last_error());
    if (e2d_write_field_plt(s, m, (out + "/unresult.plt").c_str()) ||
        e2d_write_residual_plt(s, (out + "/unresidual.plt").c_str()) ||
        e2d_write_wall_cp_plt(s, m, (out + "/unairfoilpress.plt").c_str()))
        return fail("output");
    e2d_solver_destroy(s);
    e2d_mesh_free(m);
    std::printf("All Computation's Finished!!\n");
    return rc ? 1 : 0;
}
