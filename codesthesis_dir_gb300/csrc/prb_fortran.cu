// gfortran-compatible drop-in entry points for the subroutines of
// monashubuntudir_velvor2dperiodicrbconvdir/velvor2dperiodicrbconv.f (PRB).
//
// A Fortran main program that keeps its own COMMON blocks and calls
//   cvorticity1/temperature1/heat/rhsv/poisson2/rhsu/poisson3/update
// (PRB:341-351, 363-382) links against this library instead of the Fortran
// subroutines.  Each call moves the fields the subroutine reads from the
// COMMON blocks to one process-wide device instance, runs the subroutine's
// kernels, and moves back the fields it writes, so the caller sees exactly
// the arrays the Fortran routine would have left.
//
// COMMON blocks are found through weak references to the gfortran symbols
// sol1_, sol2_, sol3_, num_, val_, radius_ (defined by the Fortran main
// program), or through gb_prb_bind_common / gb_prb_bind_radius for callers
// that are not Fortran.  Array bounds are the reference's PARAMETER values
// kr = 290, kp = 1610 unless gb_prb_bind_bounds or GB300_PRB_KR /
// GB300_PRB_KP say otherwise.
//
// The same symbols serve the rotating-annulus driver
// (iarchomedir_groke_storage_users_mpking_rotannconvvelvorplane_continueddir/
// velvor2dnewsch3.4.f, same subroutine names and COMMON blocks) once
// gb_prb_bind_variant(GB_PRB_ANNULUS) or GB300_PRB_VARIANT=annulus selects
// it; its solves then default to tolcon 1e-5 and 10000 sweeps.  mpkoks.f
// (the layer with oblique gravity, same names) is GB_PRB_OBLIQUE or
// GB300_PRB_VARIANT=oblique.
#include <stdlib.h>
#include <string.h>

#include <mutex>

#include "gbcommon.cuh"
#include "prb_internal.cuh"

extern "C" {
extern char sol1_[] __attribute__((weak));
extern char sol2_[] __attribute__((weak));
extern char sol3_[] __attribute__((weak));
extern char num_[] __attribute__((weak));
extern char val_[] __attribute__((weak));
extern char radius_[] __attribute__((weak));
}

int gb_prb_create_ex(const gb_prb_params *p, double dr, double dp, gb_prb **out, int *nlev_out);

namespace {

struct NumBlock {  // COMMON /num/ dt,dr,dz,dp,nr,nz,np (PRB:74)
    double dt, dr, dz, dp;
    int nr, nz, np;
};
struct ValBlock {  // COMMON /val/ Ra,Re,Ptl,Gr (PRB:68)
    double Ra, Re, Ptl, Gr;
};

struct DropIn {
    std::mutex mu;
    gb_prb *ctx = nullptr;
    int kr = 290, kp = 1610;
    int smoother = GB_SMOOTHER_LEX;
    int variant = GB_PRB_LAYER;
    bool tol_bound = false;   // gb_prb_bind_tolerance called: keep its values
    double tolcon = 2e-6;
    int maxsweeps = 500;
    double *sol1 = nullptr, *sol2 = nullptr, *sol3 = nullptr;
    NumBlock *num = nullptr;
    ValBlock *val = nullptr;
    double *radius = nullptr;   // COMMON /radius/ r0, rmax
    int last_status = GB_OK, last_sweeps = 0;
    bool env_read = false;
};

DropIn &g()
{
    static DropIn d;
    if (!d.env_read) {
        d.env_read = true;
        if (const char *s = getenv("GB300_PRB_KR")) d.kr = atoi(s);
        if (const char *s = getenv("GB300_PRB_KP")) d.kp = atoi(s);
        if (const char *s = getenv("GB300_PRB_VARIANT"))
        {
            if (strcmp(s, "annulus") == 0 || strcmp(s, "1") == 0) d.variant = GB_PRB_ANNULUS;
            if (strcmp(s, "oblique") == 0 || strcmp(s, "2") == 0) d.variant = GB_PRB_OBLIQUE;
            if (strcmp(s, "taycou") == 0 || strcmp(s, "3") == 0) d.variant = GB_PRB_TAYCOU;
            if (strcmp(s, "tank") == 0 || strcmp(s, "4") == 0) d.variant = GB_PRB_TANK;
            if (strcmp(s, "dvd") == 0 || strcmp(s, "5") == 0) d.variant = GB_PRB_DVD;
        }
    }
    return d;
}

double *sol1p() { return g().sol1 ? g().sol1 : (double *)sol1_; }
double *sol2p() { return g().sol2 ? g().sol2 : (double *)sol2_; }
double *sol3p() { return g().sol3 ? g().sol3 : (double *)sol3_; }
NumBlock *nump() { return g().num ? g().num : (NumBlock *)num_; }
ValBlock *valp() { return g().val ? g().val : (ValBlock *)val_; }
double *radiusp() { return g().radius ? g().radius : (double *)radius_; }

// Host address of field f inside the COMMON blocks.
double *common_field(int f)
{
    const size_t S = (size_t)(g().kr + 1) * (size_t)(g().kp + 1);
    double *b1 = sol1p(), *b2 = sol2p(), *b3 = sol3p();
    if (f >= GB_F_An && f <= GB_F_Cp) return b1 ? b1 + S * (f - GB_F_An) : nullptr;
    if (f >= GB_F_thn && f <= GB_F_thp) return b2 ? b2 + S * (f - GB_F_thn) : nullptr;
    if (f >= GB_F_uel && f <= GB_F_welp) return b3 ? b3 + S * (f - GB_F_uel) : nullptr;
    return nullptr;
}

int fail(int st)
{
    g().last_status = st;
    return st;
}

// Makes sure the device instance matches the sizes and spacings in /num/.
int ensure(int nr, int np, double dr, double dp)
{
    DropIn &d = g();
    if (nr + 1 > d.kr || np > d.kp) {
        gb_set_error("grid nr=%d np=%d exceeds the COMMON bounds kr=%d kp=%d", nr, np, d.kr, d.kp);
        return GB_ERR_INVALID;
    }
    const bool ann = d.variant == GB_PRB_ANNULUS || d.variant == GB_PRB_TAYCOU;
    double r0 = 0.5, rmax = 1.0, Re = 1.0;
    if (ann) {
        // the annulus multigrid coefficients depend on r0 (COMMON /radius/)
        if (!radiusp()) {
            gb_set_error("the annulus needs COMMON /radius/ r0,rmax (radius_ or gb_prb_bind_radius)");
            return GB_ERR_INVALID;
        }
        r0 = radiusp()[0];
        rmax = radiusp()[1];
        if (valp() && valp()->Re != 0.0) Re = valp()->Re;
    }
    if (d.ctx && d.ctx->p.nr == nr && d.ctx->p.np == np && d.ctx->dev.dr == dr && d.ctx->dev.dp == dp &&
        d.ctx->p.variant == d.variant && (!ann || (d.ctx->p.r0 == r0 && d.ctx->p.rmax == rmax)))
        return GB_OK;
    if (d.ctx) gb_prb_destroy(d.ctx);
    d.ctx = nullptr;
    gb_prb_params p;
    if (ann) {
        if (d.variant == GB_PRB_TAYCOU) gb_prb_default_params_taycou(&p, nr, np);
        else gb_prb_default_params_annulus(&p, nr, np);
        p.r0 = r0;
        p.rmax = rmax;
        p.Re = Re;
    } else if (d.variant == GB_PRB_TANK) {
        gb_prb_default_params_tank(&p, nr, np);
    } else if (d.variant == GB_PRB_DVD) {
        gb_prb_default_params_dvd(&p, nr, np);
    } else {
        gb_prb_default_params(&p, nr, np);
        p.variant = d.variant;   // GB_PRB_LAYER or GB_PRB_OBLIQUE
    }
    p.smoother = d.smoother;
    if (d.tol_bound) {
        p.tolcon = d.tolcon;
        p.maxsweeps = d.maxsweeps;
    }
    return gb_prb_create_ex(&p, dr, dp, &d.ctx, nullptr);
}

int ensure_from_common()
{
    NumBlock *n = nump();
    if (!n || !sol1p() || !sol2p() || !sol3p() || !valp()) {
        gb_set_error("COMMON blocks /num/ /sol1/ /sol2/ /sol3/ /val/ are not bound");
        return GB_ERR_INVALID;
    }
    int st = ensure(n->nr, n->np, n->dr, n->dp);
    if (st != GB_OK) return st;
    gb_prb *h = g().ctx;
    h->p.dt = n->dt;
    h->p.Ra = valp()->Ra;
    h->p.Pr = valp()->Ptl;
    if (h->p.variant == GB_PRB_TAYCOU) h->p.Ta = valp()->Gr;   // velvor2dtaycouheat.f:106-109: Gr holds Ta
    if (h->p.variant == GB_PRB_ANNULUS || h->p.variant == GB_PRB_TAYCOU) {
        h->p.Re = valp()->Re;
        h->p.r0 = radiusp()[0];
        h->p.rmax = radiusp()[1];
    }
    return GB_OK;
}

int up(std::initializer_list<int> fields)
{
    for (int f : fields) {
        int st = gb_prb_set_field(g().ctx, f, common_field(f), g().kr + 1);
        if (st != GB_OK) return st;
    }
    return GB_OK;
}

int down(std::initializer_list<int> fields)
{
    for (int f : fields) {
        int st = gb_prb_get_field(g().ctx, f, common_field(f), g().kr + 1);
        if (st != GB_OK) return st;
    }
    return GB_OK;
}

void cvort(int first)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up({GB_F_C, GB_F_Cp, GB_F_th, GB_F_uel, GB_F_vel, GB_F_A, GB_F_B, GB_F_An, GB_F_Bn, GB_F_Cn, GB_F_Ap});
    if (st == GB_OK) st = gb_prb_cvorticity(g().ctx, first);
    if (st == GB_OK) st = down({GB_F_A, GB_F_B, GB_F_An, GB_F_Bn, GB_F_Cn, GB_F_Ap, GB_F_C});
    fail(st);
}

void temp(int first)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up({GB_F_th, GB_F_thp, GB_F_uel, GB_F_vel, GB_F_A, GB_F_B, GB_F_thn, GB_F_Ap});
    if (st == GB_OK) st = gb_prb_temperature(g().ctx, first);
    if (st == GB_OK) st = down({GB_F_A, GB_F_B, GB_F_thn, GB_F_Ap, GB_F_th});
    fail(st);
}

void poisson(int which, double *psi, double *psip, double *rhs, int *nr, int *np, double *dr, double *dp,
             int *nlev)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure(*nr, *np, *dr, *dp);
    if (st != GB_OK) { fail(st); return; }
    gb_prb *h = g().ctx;
    const int fpsi = which == 2 ? GB_F_vel : GB_F_uel;
    const int fpsip = which == 2 ? GB_F_velp : GB_F_uelp;
    const int frhs = which == 2 ? GB_F_vrh : GB_F_urh;
    const int ld = g().kr + 1;
    if (nlev && *nlev != h->nlev) {
        gb_set_error("nlev=%d differs from the level count %d of poissoninit", *nlev, h->nlev);
        fail(GB_ERR_INVALID);
        return;
    }
    st = gb_prb_set_field(h, fpsi, psi, ld);
    if (st == GB_OK) st = gb_prb_set_field(h, fpsip, psip, ld);
    if (st == GB_OK) st = gb_prb_set_field(h, frhs, rhs, ld);
    int sweeps = 0, solve = GB_OK;
    if (st == GB_OK) solve = gb_prb_poisson(h, which, &sweeps);
    if (st == GB_OK && (solve == GB_OK || solve == GB_MAXSWEEPS || solve == GB_NAN)) {
        st = gb_prb_get_field(h, fpsi, psi, ld);
        if (st == GB_OK) st = gb_prb_get_field(h, fpsip, psip, ld);
    }
    g().last_sweeps = sweeps;
    fail(st != GB_OK ? st : solve);
}

}  // namespace

extern "C" {

void gb_prb_bind_bounds(int kr, int kp)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().kr = kr;
    g().kp = kp;
}

void gb_prb_bind_smoother(int smoother)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().smoother = smoother;
    if (g().ctx) g().ctx->p.smoother = smoother;
}

void gb_prb_bind_tolerance(double tolcon, int maxsweeps)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().tol_bound = true;
    g().tolcon = tolcon;
    g().maxsweeps = maxsweeps;
    if (g().ctx) {
        g().ctx->p.tolcon = tolcon;
        g().ctx->p.maxsweeps = maxsweeps;
    }
}

void gb_prb_bind_common(double *sol1, double *sol2, double *sol3, void *num, double *val)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().sol1 = sol1;
    g().sol2 = sol2;
    g().sol3 = sol3;
    g().num = (NumBlock *)num;
    g().val = (ValBlock *)val;
}

void gb_prb_bind_variant(int variant)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().variant = (variant == GB_PRB_ANNULUS || variant == GB_PRB_OBLIQUE || variant == GB_PRB_TAYCOU ||
                   variant == GB_PRB_TANK || variant == GB_PRB_DVD)
                      ? variant
                      : GB_PRB_LAYER;
}

void gb_prb_bind_radius(double *radius)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().radius = radius;
}

int gb_prb_last_status(void) { return g().last_status; }
int gb_prb_last_sweeps(void) { return g().last_sweeps; }

void poissoninit_(int *nr, int *nz, int *np, double *dr, double *dz, double *dp, int *nlev)
{
    (void)nz;
    (void)dz;
    std::lock_guard<std::mutex> lk(g().mu);
    *nlev = prb_mg_levels(*nr, g().variant);
    int st = ensure(*nr, *np, *dr, *dp);
    fail(st);
}

void poisson2_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev)
{
    (void)nz;
    (void)dz;
    poisson(2, psi, psip, rhs, nr, np, dr, dp, nlev);
}

void poisson3_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev)
{
    (void)nz;
    (void)dz;
    poisson(3, psi, psip, rhs, nr, np, dr, dp, nlev);
}

void cvorticity1_(void) { cvort(1); }
void cvorticity_(void) { cvort(0); }
void temperature1_(void) { temp(1); }
void temperature_(void) { temp(0); }

void heat_(double *trans1, double *trans2)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up({GB_F_th});
    if (st == GB_OK) st = gb_prb_heat(g().ctx, trans1, trans2);
    fail(st);
}

void update_(void)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up({GB_F_wel, GB_F_vel, GB_F_Cn, GB_F_C, GB_F_Cp, GB_F_th, GB_F_thp, GB_F_thn, GB_F_Bn});
    long long clamps = 0;
    if (st == GB_OK) st = gb_prb_update(g().ctx, &clamps);
    if (st == GB_OK) st = down({GB_F_Bn, GB_F_Cn, GB_F_Cp, GB_F_C, GB_F_thp, GB_F_thn, GB_F_th});
    // the Taylor-Couette update also sets the moving wall's v (velvor2dtaycouheat.f:1587)
    if (st == GB_OK && g().ctx->p.variant == GB_PRB_TAYCOU) st = down({GB_F_vel});
    for (long long i = 0; i < clamps && i < 16; ++i) printf(" WARNING! Temp damped\n");
    fail(st);
}

void rhsv_(double *vrh)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up({GB_F_Cn});
    if (st == GB_OK) st = gb_prb_set_field(g().ctx, GB_F_vrh, vrh, g().kr + 1);
    if (st == GB_OK) st = gb_prb_rhsv(g().ctx);
    if (st == GB_OK) st = gb_prb_get_field(g().ctx, GB_F_vrh, vrh, g().kr + 1);
    fail(st);
}

void rhsu_(double *urh)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up({GB_F_Cn});
    if (st == GB_OK) st = gb_prb_set_field(g().ctx, GB_F_urh, urh, g().kr + 1);
    if (st == GB_OK) st = gb_prb_rhsu(g().ctx);
    if (st == GB_OK) st = gb_prb_get_field(g().ctx, GB_F_urh, urh, g().kr + 1);
    fail(st);
}

}  // extern "C"
