// les_reference_api.h -- the les-model host interface, served by the GB300
// library.
//
// A caller of les-model (its step loop, checkpoint, VTK and statistics code)
// includes the reference's own field.h and pressure.h and links
// les-model_gb300/libles_shim.so instead of pressure.cpp and the step
// functions of main.cpp.  This header restates those declarations so that the
// shim and its tests compile without the reference tree: the types must stay
// layout- and name-compatible with src/field.h:6-48 and src/pressure.h:11-29,
// and the functions keep the signatures of src/pressure.h:31-63 and the
// prototypes of src/main.cpp:20-29 (the interface has to be identical for the
// drop-in to link; see the shim for the semantics of each call).
#ifndef LES_REFERENCE_API_H
#define LES_REFERENCE_API_H

#include <vector>

#ifndef LES_MODEL_FIELD_H
#define LES_MODEL_FIELD_H
struct Mesh {
    int nx, ny, nz;
    double dx, dy, dz;
};

struct Field {
    int nx, ny, nz;
    std::vector<double> u, v, w;
    std::vector<double> u_new, v_new, w_new;
    std::vector<double> p;
    std::vector<double> p_rhs;
    std::vector<double> nu_t;
    std::vector<bool> is_solid;
    Field() : nx(0), ny(0), nz(0) {}
    Field(int a, int b, int c)
        : nx(a), ny(b), nz(c), u(size_t(a) * b * c, 0.0), v(size_t(a) * b * c, 0.0),
          w(size_t(a) * b * c, 0.0), u_new(size_t(a) * b * c, 0.0), v_new(size_t(a) * b * c, 0.0),
          w_new(size_t(a) * b * c, 0.0), p(size_t(a) * b * c, 0.0), p_rhs(size_t(a) * b * c, 0.0),
          nu_t(size_t(a) * b * c, 0.0), is_solid(size_t(a) * b * c, false)
    {
    }
    int idx(int i, int j, int k) const { return i * ny * nz + j * nz + k; }
};

struct Stress {
    std::vector<double> tau_xx, tau_xy, tau_xz;
    std::vector<double> tau_yy, tau_yz, tau_zz;
    Stress(int n) : tau_xx(n, 0.0), tau_xy(n, 0.0), tau_xz(n, 0.0), tau_yy(n, 0.0), tau_yz(n, 0.0), tau_zz(n, 0.0) {}
};
#endif

#ifndef PRESSURE_H
#define PRESSURE_H
using Vector = std::vector<double>;

struct StencilMatrix {
    Vector A_c, A_n, A_s, A_e, A_w, A_t, A_b;
    StencilMatrix(int n)
        : A_c(n, 0.0), A_n(n, 0.0), A_s(n, 0.0), A_e(n, 0.0), A_w(n, 0.0), A_t(n, 0.0), A_b(n, 0.0)
    {
    }
};

void apply_pressure_BCs(Field& f, const Mesh& m);
void solve_pressure_jacobi(Field& f, const Mesh& m, double dt, double rho);
void solve_pressure_GS(Field& f, const Mesh& m, double dt, double rho, int maxIter = 200);
int solve_pressure_pcg(const StencilMatrix& A, const Vector& b, Vector& x, const Field& field, int max_iter,
                       double tol);
void calculate_divergence(Vector& divergence, const Field& f, const Mesh& m, double dt, double rho);
void build_stencil(StencilMatrix& A, const Field& field, const Mesh& m);
void build_b_vector(Vector& b, const Vector& divergence, const Field& field, const Mesh& m);
void fast_apply_laplacian(Vector& q, const Vector& p, const StencilMatrix& A, const Field& field);
void apply_jacobi_preconditioner(Vector& z, const Vector& r, const StencilMatrix& A);
void apply_ic_preconditioner(Vector& z, const Vector& r, const StencilMatrix& L, const Field& field);
void build_ic_preconditioner(StencilMatrix& L, const StencilMatrix& A, const Field& field, const Mesh& m);
int solve_pressure_pcg_chebyshev(const StencilMatrix& A, const Vector& b, Vector& x, const Field& field,
                                 double lambda_min, double lambda_max, int poly_degree = 5, int maxIter = 100,
                                 double tol = 1e-6);
void apply_chebyshev_preconditioner(Vector& z, const Vector& r, const StencilMatrix& A, const Field& field,
                                    double lambda_min, double lambda_max, int poly_degree = 5);
double estimate_lambda_max(const StencilMatrix& A, const Field& field, int n_iter = 20);
void parallel_axpy(Vector& v_out, double a, const Vector& v_in);
double parallel_norm(const Vector& v);
double parallel_dot(const Vector& v1, const Vector& v2);
void parallel_saxpy(Vector& v_out, double a, const Vector& v_in1, double b, const Vector& v_in2);
void parallel_copy(Vector& v_out, const Vector& v_in);
#endif

// Step functions the reference defines in src/main.cpp (prototypes :20-29).
double compute_adaptive_dt(const Field& field, const Mesh& mesh, double nu);
void compute_sgs_stress(Field& f, Stress& sgs, const Mesh& m);
void apply_nut_BCs(Field& f, const Mesh& m);
void solve_momentum(Field& f, const Mesh& m, double dt, double nu);
void apply_velocity_BCs(Field& f, const Mesh& m);
void correct_velocity(Field& f, const Mesh& m, double dt, double rho);

// ---- GB300 additions (no reference counterpart) --------------------------
namespace les_shim {
// Device used for new contexts (default 0, or the LES_DEVICE environment
// variable).
void set_device(int device);
// Drops every cached device context and matrix (call after changing a
// StencilMatrix in place: the shim caches matrices by address).
void reset();
// Device status of the last failing call (the reference API has no error
// returns; a failing call throws std::runtime_error with this text).
const char* last_error();
}  // namespace les_shim

#endif
