// shim_loop.cpp -- the step loop of les-model src/main.cpp:108-144 (without
// the prompt, I/O and statistics) written against the reference API, linked
// to libles_shim.so.  Test driver for tests/test_gpu_shim.py.
//
//   shim_loop in.bin out.bin nx ny nz h solver nsteps
//   solver: 0 as-shipped PCG, 3 Chebyshev PCG, 4 Jacobi, 5 GS-SOR
// in.bin: u, v, w (N doubles each) then is_solid (N bytes).
// out.bin: u, v, w, u_new, v_new, w_new, p, p_rhs, nu_t (N doubles each).
// stdout: one line per step "step <s> dt <dt> iters <n>", then BLAS-1 checks.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "les_reference_api.h"

int main(int argc, char** argv)
{
    if (argc < 9) return 2;
    const int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]), nz = std::atoi(argv[5]);
    const double h = std::atof(argv[6]);
    const int solver = std::atoi(argv[7]), nsteps = std::atoi(argv[8]);
    const int n = nx * ny * nz;
    Mesh mesh{nx, ny, nz, h, h, h};
    Field field(nx, ny, nz);
    Stress sgs(n);
    std::vector<unsigned char> solid(n);
    FILE* fi = std::fopen(argv[1], "rb");
    if (!fi) return 3;
    size_t got = std::fread(field.u.data(), 8, n, fi) + std::fread(field.v.data(), 8, n, fi) +
                 std::fread(field.w.data(), 8, n, fi) + std::fread(solid.data(), 1, n, fi);
    std::fclose(fi);
    if (got != (size_t)4 * n) return 4;

    // setup in src/main.cpp:64-81 order: A, L and lambda_max before the mask
    StencilMatrix A(n);
    build_stencil(A, field, mesh);
    StencilMatrix L(n);
    build_ic_preconditioner(L, A, field, mesh);
    const double lambda_max = estimate_lambda_max(A, field, 20);
    const double lambda_min = 3.0 * M_PI * M_PI;
    for (int i = 0; i < n; ++i) field.is_solid[i] = solid[i] != 0;
    const double rho = 1.2, nu = 1.0e-5;
    apply_velocity_BCs(field, mesh);

    for (int step = 0; step < nsteps; ++step) {
        double dt = (step == nsteps - 1) ? compute_adaptive_dt(field, mesh, nu) : 1e-4;
        compute_sgs_stress(field, sgs, mesh);
        apply_nut_BCs(field, mesh);
        solve_momentum(field, mesh, dt, nu);
        apply_velocity_BCs(field, mesh);
        int iters = 0;
        if (solver == 0 || solver == 3) {
            calculate_divergence(field.p_rhs, field, mesh, dt, rho);
            Vector b(n);
            build_b_vector(b, field.p_rhs, field, mesh);
            const double tol = 1e-8 * parallel_norm(b);
            if (solver == 0) iters = solve_pressure_pcg(A, b, field.p, field, 200, tol);
            else iters = solve_pressure_pcg_chebyshev(A, b, field.p, field, lambda_min, lambda_max, 4, 200, tol);
        } else if (solver == 4) {
            solve_pressure_jacobi(field, mesh, dt, rho);
        } else {
            solve_pressure_GS(field, mesh, dt, rho, 40);
        }
        correct_velocity(field, mesh, dt, rho);
        apply_velocity_BCs(field, mesh);
        std::printf("step %d dt %.17g iters %d\n", step, dt, iters);
    }
    // BLAS-1 helpers on the final fields
    Vector a = field.u, c(n);
    parallel_axpy(a, 0.5, field.v);
    parallel_saxpy(c, 2.0, field.w, -3.0, field.p);
    std::printf("lambda %.17g\n", lambda_max);
    std::printf("dot %.17g norm %.17g\n", parallel_dot(field.u, field.v), parallel_norm(field.p));
    std::printf("axpy %.17g saxpy %.17g\n", a[n / 2], c[n / 3]);

    FILE* fo = std::fopen(argv[2], "wb");
    if (!fo) return 5;
    const std::vector<double>* out[9] = {&field.u, &field.v, &field.w, &field.u_new, &field.v_new,
                                         &field.w_new, &field.p, &field.p_rhs, &field.nu_t};
    for (auto* v : out) std::fwrite(v->data(), 8, n, fo);
    std::fclose(fo);
    return 0;
}
