// gfortran-compatible drop-in entry points for the subroutines of rot3dmg.f
// (the 3D rotating annulus), over the gb_r3d_* context API of
// libgb300conv.so.  Built as its own library, libgb300r3d.so, because the
// names clash with the 2D drivers' drop-ins.  Host code only.
//
// Each call binds the caller's COMMON blocks (weak references to gfortran's
// sol1_ ... radius_, or gb_r3d_bind_common), makes sure the process-wide
// device instance matches /num/, /val/ and /radius/ (recreating it when
// they change), copies the fields the Fortran routine reads to the device,
// runs the routine, and copies back the fields it writes.  The device
// kernels write only what the reference writes, so the untouched parts of
// every array round-trip unchanged.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <initializer_list>
#include <mutex>

#define GB300_NO_PRB_DROPIN
#include "gb300_convection.h"
#include "gb300_r3d_fortran.h"

extern "C" {
extern char sol1_[] __attribute__((weak));
extern char sol2_[] __attribute__((weak));
extern char sol3_[] __attribute__((weak));
extern char num_[] __attribute__((weak));
extern char val_[] __attribute__((weak));
extern char radius_[] __attribute__((weak));
}

namespace {

struct NumBlock {  // COMMON /num/ dt,dr,dz,dp,nr,nz,np (rot3dmg.f:40)
    double dt, dr, dz, dp;
    int nr, nz, np;
};
struct ValBlock {  // COMMON /val/ Ra,Re,Ptl,Gr (rot3dmg.f:36)
    double Ra, Re, Ptl, Gr;
};

struct DropIn {
    std::mutex mu;
    gb_r3d *ctx = nullptr;
    gb_r3d_params cur;
    double cur_dr = 0, cur_dz = 0, cur_dp = 0;
    int kr = 33, kz = 33, kp = 160;
    int smoother = GB_SMOOTHER_LEX, precision = GB_PRB_FP64;
    int variant = GB_R3D_VERTICAL;
    bool tol_bound = false;
    double tolcon = 1e-5;
    int maxsweeps = 500;
    double *sol1 = nullptr, *sol2 = nullptr, *sol3 = nullptr, *radius = nullptr;
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
        if (const char *s = getenv("GB300_R3D_KR")) d.kr = atoi(s);
        if (const char *s = getenv("GB300_R3D_KZ")) d.kz = atoi(s);
        if (const char *s = getenv("GB300_R3D_KP")) d.kp = atoi(s);
        if (const char *s = getenv("GB300_R3D_VARIANT"))
            if (strcmp(s, "horizontal") == 0 || strcmp(s, "1") == 0) d.variant = GB_R3D_HORIZONTAL;
    }
    return d;
}

double *sol1p() { return g().sol1 ? g().sol1 : (double *)sol1_; }
double *sol2p() { return g().sol2 ? g().sol2 : (double *)sol2_; }
double *sol3p() { return g().sol3 ? g().sol3 : (double *)sol3_; }
NumBlock *nump() { return g().num ? g().num : (NumBlock *)num_; }
ValBlock *valp() { return g().val ? g().val : (ValBlock *)val_; }
double *radiusp() { return g().radius ? g().radius : (double *)radius_; }

size_t field_size() { return (size_t)(g().kr + 1) * (size_t)(g().kz + 1) * (size_t)(g().kp + 1); }

// Host address of field f inside the COMMON blocks (rot3dmg.f:37-39).
double *common_field(int f)
{
    const size_t S = field_size();
    double *b1 = sol1p(), *b2 = sol2p(), *b3 = sol3p();
    if (f >= GB_R_An && f <= GB_R_Cp) return b1 ? b1 + S * (f - GB_R_An) : nullptr;
    if (f >= GB_R_thn && f <= GB_R_thp) return b2 ? b2 + S * (f - GB_R_thn) : nullptr;
    if (f >= GB_R_uel && f <= GB_R_welp) return b3 ? b3 + S * (f - GB_R_uel) : nullptr;
    return nullptr;
}

int fail(int st)
{
    g().last_status = st;
    return st;
}

// The device instance for grid (nr, nz, np) with the given spacings and the
// physics in /val/, /num/ and /radius/; recreated whenever any of them
// differs from the instance's.
int ensure(int nr, int nz, int np, double dr, double dz, double dp)
{
    DropIn &d = g();
    if (nr + 1 > d.kr || nz + 1 > d.kz || np > d.kp) {
        fprintf(stderr, "gb300 r3d: grid %d x %d x %d exceeds the COMMON bounds kr=%d kz=%d kp=%d\n", nr, nz, np,
                d.kr, d.kz, d.kp);
        return GB_ERR_INVALID;
    }
    if (!valp() || !radiusp()) return GB_ERR_INVALID;
    gb_r3d_params p;
    gb_r3d_default_params(&p, nr, nz, np);
    p.r0 = radiusp()[0];
    p.rmax = radiusp()[1];
    p.zmax = dz * (double)nz;   // used for nothing the routines compute
    if (nump()) p.dt = nump()->dt;
    p.Ra = valp()->Ra;
    p.Re = valp()->Re;
    p.Gr = valp()->Gr;
    p.Pr = valp()->Ptl;
    p.smoother = d.smoother;
    p.precision = d.precision;
    p.variant = d.variant;
    if (d.variant == GB_R3D_HORIZONTAL) p.tolcon = 1e-6;   // rot3dmghor.f:1599, :1798, :2051
    if (d.tol_bound) {
        p.tolcon = d.tolcon;
        p.maxsweeps = d.maxsweeps;
    }
    if (d.ctx && memcmp(&p, &d.cur, sizeof(p)) == 0 && dr == d.cur_dr && dz == d.cur_dz && dp == d.cur_dp)
        return GB_OK;
    if (d.ctx) gb_r3d_destroy(d.ctx);
    d.ctx = nullptr;
    int nlev = 0;
    const int st = gb_r3d_create_spacing(&p, dr, dz, dp, &d.ctx, &nlev);
    if (st != GB_OK) {
        fprintf(stderr, "gb300 r3d: %s\n", gb_last_error());
        d.ctx = nullptr;
        return st;
    }
    d.cur = p;
    d.cur_dr = dr;
    d.cur_dz = dz;
    d.cur_dp = dp;
    return GB_OK;
}

int ensure_from_common()
{
    NumBlock *n = nump();
    if (!n || !sol1p() || !sol2p() || !sol3p() || !valp() || !radiusp()) {
        fprintf(stderr, "gb300 r3d: COMMON blocks /num/ /sol1/ /sol2/ /sol3/ /val/ /radius/ are not bound\n");
        return GB_ERR_INVALID;
    }
    return ensure(n->nr, n->nz, n->np, n->dr, n->dz, n->dp);
}

int up(std::initializer_list<int> fields)
{
    for (int f : fields) {
        const int st = gb_r3d_set_field(g().ctx, f, common_field(f), g().kr + 1, g().kz + 1);
        if (st != GB_OK) return st;
    }
    return GB_OK;
}

int down(std::initializer_list<int> fields)
{
    for (int f : fields) {
        const int st = gb_r3d_get_field(g().ctx, f, common_field(f), g().kr + 1, g().kz + 1);
        if (st != GB_OK) return st;
    }
    return GB_OK;
}

// Transport routine: upload what it reads (and the field it writes, so that
// the parts it leaves alone come back unchanged), run, download.
void transport(int (*fn)(gb_r3d *), int out, std::initializer_list<int> in)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up(in);
    if (st == GB_OK) st = up({out});
    if (st == GB_OK) st = fn(g().ctx);
    if (st == GB_OK) st = down({out});
    fail(st);
}

void rhs(int (*fn)(gb_r3d *), int field, double *arr, std::initializer_list<int> in)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up(in);
    if (st == GB_OK) st = gb_r3d_set_field(g().ctx, field, arr, g().kr + 1, g().kz + 1);
    if (st == GB_OK) st = fn(g().ctx);
    if (st == GB_OK) st = gb_r3d_get_field(g().ctx, field, arr, g().kr + 1, g().kz + 1);
    fail(st);
}

void poisson(int which, double *psi, double *psip, double *prhs, int *nr, int *nz, int *np, double *dr, double *dz,
             double *dp, int *nlev)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure(*nr, *nz, *np, *dr, *dz, *dp);
    if (st != GB_OK) { fail(st); return; }
    gb_r3d *h = g().ctx;
    const int fpsi = which == 1 ? GB_R_wel : which == 2 ? GB_R_vel : GB_R_uel;
    const int fpsip = which == 1 ? GB_R_welp : which == 2 ? GB_R_velp : GB_R_uelp;
    const int frhs = which == 1 ? GB_R_wrh : which == 2 ? GB_R_vrh : GB_R_urh;
    const int l1 = g().kr + 1, l2 = g().kz + 1;
    st = gb_r3d_set_field(h, fpsi, psi, l1, l2);
    if (st == GB_OK) st = gb_r3d_set_field(h, fpsip, psip, l1, l2);
    if (st == GB_OK) st = gb_r3d_set_field(h, frhs, prhs, l1, l2);
    int sweeps = 0, solve = GB_OK;
    if (st == GB_OK) solve = gb_r3d_poisson(h, which, &sweeps);
    if (st == GB_OK && solve == GB_OK) {
        st = gb_r3d_get_field(h, fpsi, psi, l1, l2);
        if (st == GB_OK) st = gb_r3d_get_field(h, fpsip, psip, l1, l2);
    }
    (void)nlev;
    g().last_sweeps = sweeps;
    fail(st != GB_OK ? st : solve);
}

// poissoninit's level rule (rot3dmg.f:1172-1192).
int levels(int nr, int nz)
{
    int nlev = 0, itest = nr, itest2 = nr, jtest = nz, jtest2 = nz;
    for (int i = 2; i <= 8; ++i) {
        itest /= 2;
        jtest /= 2;
        if (itest * 2 - itest2 == 0 && jtest * 2 - jtest2 == 0) {
            if (itest2 >= 4 && jtest2 >= 4) nlev++;
            itest2 = itest;
            jtest2 = jtest;
        } else {
            break;
        }
    }
    return nlev > 4 ? 4 : nlev;
}

}  // namespace

extern "C" {

void gb_r3d_bind_bounds(int kr, int kz, int kp)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().kr = kr;
    g().kz = kz;
    g().kp = kp;
}

void gb_r3d_bind_common(double *sol1, double *sol2, double *sol3, void *num, double *val, double *radius)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().sol1 = sol1;
    g().sol2 = sol2;
    g().sol3 = sol3;
    g().num = (NumBlock *)num;
    g().val = (ValBlock *)val;
    g().radius = radius;
}

void gb_r3d_bind_smoother(int smoother)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().smoother = smoother;
}

void gb_r3d_bind_variant(int variant)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().variant = variant == GB_R3D_HORIZONTAL ? GB_R3D_HORIZONTAL : GB_R3D_VERTICAL;
}

void gb_r3d_bind_precision(int precision)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().precision = precision;
}

void gb_r3d_bind_tolerance(double tolcon, int maxsweeps)
{
    std::lock_guard<std::mutex> lk(g().mu);
    g().tol_bound = true;
    g().tolcon = tolcon;
    g().maxsweeps = maxsweeps;
}

int gb_r3d_last_status(void) { return g().last_status; }
int gb_r3d_last_sweeps(void) { return g().last_sweeps; }

void poissoninit_(int *nr, int *nz, int *np, double *dr, double *dz, double *dp, int *nlev)
{
    std::lock_guard<std::mutex> lk(g().mu);
    *nlev = levels(*nr, *nz);
    fail(ensure(*nr, *nz, *np, *dr, *dz, *dp));
}

void poisson1_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev)
{
    poisson(1, psi, psip, rhs, nr, nz, np, dr, dz, dp, nlev);
}

void poisson2_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev)
{
    poisson(2, psi, psip, rhs, nr, nz, np, dr, dz, dp, nlev);
}

void poisson3_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev)
{
    poisson(3, psi, psip, rhs, nr, nz, np, dr, dz, dp, nlev);
}

void avorticity_(void)
{
    transport(gb_r3d_avorticity, GB_R_An,
              {GB_R_A, GB_R_Ap, GB_R_B, GB_R_C, GB_R_th, GB_R_uel, GB_R_vel, GB_R_wel});
}

void bvorticity_(void)
{
    transport(gb_r3d_bvorticity, GB_R_Bn,
              {GB_R_A, GB_R_B, GB_R_Bp, GB_R_C, GB_R_th, GB_R_uel, GB_R_vel, GB_R_wel});
}

void cvorticity_(void)
{
    transport(gb_r3d_cvorticity, GB_R_Cn,
              {GB_R_A, GB_R_B, GB_R_C, GB_R_Cp, GB_R_th, GB_R_uel, GB_R_vel, GB_R_wel});
}

void temperature_(void)
{
    transport(gb_r3d_temperature, GB_R_thn, {GB_R_th, GB_R_thp, GB_R_uel, GB_R_vel, GB_R_wel});
}

// rot3dmg.f calls heat(trans1); rot3dmghor.f calls heat(trans1, trans2),
// and only the horizontal variant reads the second argument.
void heat_(double *trans1, double *trans2)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK) st = up({GB_R_th});
    if (st == GB_OK)
        st = g().variant == GB_R3D_HORIZONTAL ? gb_r3d_heat2(g().ctx, trans1, trans2) : gb_r3d_heat(g().ctx, trans1);
    fail(st);
}

void update_(void)
{
    std::lock_guard<std::mutex> lk(g().mu);
    int st = ensure_from_common();
    if (st == GB_OK)
        st = up({GB_R_uel, GB_R_vel, GB_R_wel, GB_R_An, GB_R_Bn, GB_R_Cn, GB_R_thn, GB_R_A, GB_R_B, GB_R_C, GB_R_th});
    if (st == GB_OK) st = gb_r3d_update(g().ctx);
    if (st == GB_OK)
        st = down({GB_R_An, GB_R_Bn, GB_R_Cn, GB_R_thn, GB_R_Ap, GB_R_A, GB_R_Bp, GB_R_B, GB_R_Cp, GB_R_C, GB_R_thp,
                   GB_R_th});
    fail(st);
}

void rhsw_(double *wrh) { rhs(gb_r3d_rhsw, GB_R_wrh, wrh, {GB_R_An, GB_R_Bn}); }
void rhsv_(double *vrh) { rhs(gb_r3d_rhsv, GB_R_vrh, vrh, {GB_R_An, GB_R_Cn}); }
void rhsu_(double *urh) { rhs(gb_r3d_rhsu, GB_R_urh, urh, {GB_R_Bn, GB_R_Cn, GB_R_wel}); }

}  // extern "C"
