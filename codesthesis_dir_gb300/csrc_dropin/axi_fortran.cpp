// gfortran-compatible drop-in entry points for the subroutines of rotann2.f
// (the axisymmetric rotating annulus), over the gb_axi_* context API of
// libgb300conv.so.  Built as its own library, libgb300axi.so, because the
// names clash with the 2D and 3D drivers' drop-ins.  Host code only.
//
// Each call binds the caller's COMMON blocks (weak references to gfortran's
// sol1_, sol2_, num_, val_, radius_, or gb_axi_bind_common), makes sure the
// process-wide device instance matches /num/, /val/ and /radius/ (recreating
// it when they change), copies the ten fields of /sol1/ and /sol2/ to the
// device, runs the routine, and copies them back.  The device kernels write
// only what the reference writes, so every field the routine leaves alone
// round-trips unchanged.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>

#define GB300_NO_PRB_DROPIN
#include "gb300_axi_fortran.h"
#include "gb300_convection.h"

extern "C" {
extern char sol1_[] __attribute__((weak));
extern char sol2_[] __attribute__((weak));
extern char num_[] __attribute__((weak));
extern char val_[] __attribute__((weak));
extern char radius_[] __attribute__((weak));
}

namespace {

struct NumBlock {  // COMMON /num/ dr,dz,nr,nz,dt (rotann2.f:22)
    double dr, dz;
    int nr, nz;
    double dt;
};
struct ValBlock {  // COMMON /val/ cf1,cf2,cf3,cf4,Ra,Re,Ptl (rotann2.f:19)
    double cf1, cf2, cf3, cf4, Ra, Re, Ptl;
};

struct DropIn {
    std::mutex mu;
    gb_axi *ctx = nullptr;
    gb_axi_params cur;
    double cur_dr = 0, cur_dz = 0;
    int nrmax = 128, nzmax = 128;   // rotann2.f:9
    int smoother = GB_SMOOTHER_LEX, precision = GB_PRB_FP64;
    bool tol_bound = false;
    double tolcon = 1e-6;
    int maxsweeps = 10000;
    double *sol1 = nullptr, *sol2 = nullptr, *radius = nullptr;
    NumBlock *num = nullptr;
    ValBlock *val = nullptr;
    int last_status = GB_OK, last_sweeps = 0;
    bool env_read = false;
};

DropIn &g()
{
    static DropIn d;
    if (!d.env_read) {
        d.env_read = true;
        if (const char *s = getenv("GB300_AXI_NRMAX")) d.nrmax = atoi(s);
        if (const char *s = getenv("GB300_AXI_NZMAX")) d.nzmax = atoi(s);
    }
    return d;
}

double *sol1p() { return g().sol1 ? g().sol1 : (double *)sol1_; }
double *sol2p() { return g().sol2 ? g().sol2 : (double *)sol2_; }
NumBlock *nump() { return g().num ? g().num : (NumBlock *)num_; }
ValBlock *valp() { return g().val ? g().val : (ValBlock *)val_; }
double *radiusp() { return g().radius ? g().radius : (double *)radius_; }

size_t field_size() { return (size_t)(g().nrmax + 1) * (size_t)(g().nzmax + 1); }

// Host address of field f in the COMMON blocks (rotann2.f:20-21).
double *common_field(int f)
{
    const size_t S = field_size();
    if (f <= GB_A_velp) return sol1p() ? sol1p() + S * (size_t)f : nullptr;
    return sol2p() ? sol2p() + S * (size_t)(f - GB_A_thetan) : nullptr;
}

int fail(int st)
{
    g().last_status = st;
    return st;
}

// The device instance for grid (nr, nz) with the caller's spacings and the
// physics in /num/, /val/ and /radius/; recreated whenever any differs.
int ensure(int nr, int nz, double dr, double dz)
{
    DropIn &d = g();
    if (nr > d.nrmax || nz > d.nzmax) {
        fprintf(stderr, "gb300 axi: grid %d x %d exceeds the array bounds nrmax=%d nzmax=%d\n", nr, nz, d.nrmax,
                d.nzmax);
        return GB_ERR_INVALID;
    }
    if (!valp() || !radiusp() || !nump()) return GB_ERR_INVALID;
    gb_axi_params p;
    gb_axi_default_params(&p, nr, nz);
    p.dt = nump()->dt;
    p.r0 = radiusp()[0];
    p.rmax = p.r0 + dr * (double)nr;   // the routines see only r0 and dr
    p.zmax = dz * (double)nz;
    p.Ra = valp()->Ra;
    p.Re = valp()->Re;
    p.Pr = valp()->Ptl;
    p.smoother = d.smoother;
    p.precision = d.precision;
    if (d.tol_bound) {
        p.tolcon = d.tolcon;
        p.maxsweeps = d.maxsweeps;
    }
    if (d.ctx && memcmp(&p, &d.cur, sizeof(p)) == 0 && dr == d.cur_dr && dz == d.cur_dz) return GB_OK;
    if (d.ctx) gb_axi_destroy(d.ctx);
    d.ctx = nullptr;
    const int st = gb_axi_create_spacing(&p, dr, dz, &d.ctx, nullptr);
    if (st != GB_OK) {
        fprintf(stderr, "gb300 axi: %s\n", gb_last_error());
        d.ctx = nullptr;
        return st;
    }
    d.cur = p;
    d.cur_dr = dr;
    d.cur_dz = dz;
    return GB_OK;
}

int ensure_from_common()
{
    NumBlock *n = nump();
    if (!n || !sol1p() || !sol2p() || !valp() || !radiusp()) {
        fprintf(stderr, "gb300 axi: COMMON blocks /num/ /sol1/ /sol2/ /val/ /radius/ are not bound\n");
        return GB_ERR_INVALID;
    }
    return ensure(n->nr, n->nz, n->dr, n->dz);
}

int up_all()
{
    for (int f = 0; f < GB_A_COUNT; ++f) {
        const int st = gb_axi_set_field(g().ctx, f, common_field(f), g().nrmax + 1);
        if (st != GB_OK) return st;
    }
    return GB_OK;
}

int down_all()
{
    for (int f = 0; f < GB_A_COUNT; ++f) {
        const int st = gb_axi_get_field(g().ctx, f, common_field(f), g().nrmax + 1);
        if (st != GB_OK) return st;
    }
    return GB_OK;
}

void routine(int (*fn)(gb_axi *))
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up_all();
    if (st == GB_OK) st = fn(g().ctx);
    if (st == GB_OK) st = down_all();
    fail(st);
}

}  // namespace

extern "C" {

void gb_axi_bind_bounds(int nrmax, int nzmax)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().nrmax = nrmax;
    g().nzmax = nzmax;
}

void gb_axi_bind_common(double *sol1, double *sol2, void *num, double *val, double *radius)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().sol1 = sol1;
    g().sol2 = sol2;
    g().num = (NumBlock *)num;
    g().val = (ValBlock *)val;
    g().radius = radius;
}

void gb_axi_bind_smoother(int smoother)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().smoother = smoother;
}

void gb_axi_bind_precision(int precision)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().precision = precision;
}

void gb_axi_bind_tolerance(double tolcon, int maxsweeps)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().tol_bound = true;
    g().tolcon = tolcon;
    g().maxsweeps = maxsweeps;
}

int gb_axi_last_status(void) { return g().last_status; }
int gb_axi_last_sweeps(void) { return g().last_sweeps; }

void poissoninit_(int *nr, int *nz, double *dr, double *dz)
{
    std::lock_guard<std::mutex> lk(g().mu);
    fail(ensure(*nr, *nz, *dr, *dz));
}

void vorticity_(void) { routine(gb_axi_vorticity); }
void velocity_(void) { routine(gb_axi_velocity); }
void temperature_(void) { routine(gb_axi_temperature); }
void update_(void) { routine(gb_axi_update); }

// poisson(psi, rhs): psi is the initial guess and the result (rotann2.f:632,
// :659-661); after the sweep limit the reference returns with psi untouched
// (:667), and so does this.
void poisson_(double *psi, double *rhs)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up_all();
    const int ld = g().nrmax + 1;
    if (st == GB_OK) st = gb_axi_set_field(g().ctx, GB_A_phi, psi, ld);
    if (st == GB_OK) st = gb_axi_set_field(g().ctx, GB_A_omegn, rhs, ld);
    int sweeps = 0, solve = GB_OK;
    if (st == GB_OK) solve = gb_axi_poisson(g().ctx, &sweeps);
    if (st == GB_OK && solve == GB_OK) st = gb_axi_get_field(g().ctx, GB_A_phi, psi, ld);
    g().last_sweeps = sweeps;
    fail(st != GB_OK ? st : solve);
}

void heat_(double *trans)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up_all();
    if (st == GB_OK) st = gb_axi_heat(g().ctx, trans);
    fail(st);
}

}  // extern "C"
