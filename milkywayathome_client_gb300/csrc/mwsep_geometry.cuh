/* mwsep_geometry.cuh -- survey geometry and convolution-table formulas,
 * usable on the host (glibc libm) and on the device (CUDA libm).
 *
 * Each function restates the reference function cited beside it in the
 * reference's association order.  Host callers compile with
 * -ffp-contract=off and device callers with -fmad=false, so no step is
 * fused.  The Sgr rotation is written in its simplified Euler-angle form
 * (the reference's entries are ratios with denominators identically one). */
#ifndef MWSEP_GEOMETRY_CUH
#define MWSEP_GEOMETRY_CUH

#include <math.h>
#include "mwsep_internal.h"

namespace mwsep {


/* atSurveyGeometry.c:87-119 (atBound, atBound2) */
MWSEP_HD inline void bound(double& a, double lo, double hi)
{
    /* The reference loops; the angles reaching here are within one turn of
     * the range, so the loops run at most twice.  Bounded for safety. */
    for (int i = 0; i < 8 && a < lo; ++i) a += 360.0;
    for (int i = 0; i < 8 && a >= hi; ++i) a -= 360.0;
}

MWSEP_HD inline void bound2(double& theta, double& phi)
{
    bound(theta, -180.0, 180.0);
    if (fabs(theta) > 90.0)
    {
        theta = 180.0 - theta;
        phi += 180;
    }
    bound(theta, -180.0, 180.0);
    bound(phi, 0.0, 360.0);
    if (fabs(theta) == 90.0) phi = 0.;
}

/* atSurveyGeometry.h:27-28 dmod */
MWSEP_HD inline double dmod(double a, double b)
{
    if (b == 0.0) return a;
    return (a * b > 0.0) ? a - b * floor(a / b) : a + b * floor(-a / b);
}

/* atSurveyGeometry.c:26-64; degree conversions evaluate as (x*pi)/180 and
 * (x*180)/pi, as the reference's macros expand. */
MWSEP_HD inline void gc_to_eq(double amu, double anu, double anode, double ainc, double& ra, double& dec)
{
    amu = amu * MW_PI / 180.0;
    anu = anu * MW_PI / 180.0;
    anode = anode * MW_PI / 180.0;
    ainc = ainc * MW_PI / 180.0;
    const double x2 = cos(amu - anode) * cos(anu);
    const double y2 = sin(amu - anode) * cos(anu);
    const double z2 = sin(anu);
    const double x1 = x2;
    const double y1 = y2 * cos(ainc) - z2 * sin(ainc);
    const double z1 = y2 * sin(ainc) + z2 * cos(ainc);
    ra = atan2(y1, x1) + anode;
    dec = asin(z1);
    ra = ra * 180.0 / MW_PI;
    dec = dec * 180.0 / MW_PI;
    bound2(dec, ra);
}

/* atSurveyGeometry.c:66-83 with slaEqgal :212-240 */
MWSEP_HD inline void eq_to_gal(double ra, double dec, double& gl, double& gb)
{
    ra = ra * MW_PI / 180.0;
    dec = dec * MW_PI / 180.0;
    const double cosb = cos(dec);
    const double v0 = cos(ra) * cosb, v1 = sin(ra) * cosb, v2 = sin(dec);
    double w;
    w = 0.0; w += -0.054875539726 * v0; w += -0.873437108010 * v1; w += -0.483834985808 * v2;
    const double x = w;
    w = 0.0; w += 0.494109453312 * v0; w += -0.444829589425 * v1; w += 0.746982251810 * v2;
    const double y = w;
    w = 0.0; w += -0.867666135858 * v0; w += -0.198076386122 * v1; w += 0.455983795705 * v2;
    const double z = w;
    const double r = sqrt(x * x + y * y);
    double dl = (r != 0.0) ? atan2(y, x) : 0.0;
    double db = (z != 0.0) ? atan2(z, r) : 0.0;
    w = dmod(dl, MW_D2PI);
    dl = (w >= 0.0) ? w : w + MW_D2PI;
    w = dmod(db, MW_D2PI);
    db = (fabs(w) < MW_PI) ? w : w - ((db < 0.0) ? -MW_D2PI : MW_D2PI);
    gl = dl * 180.0 / MW_PI;
    gb = db * 180.0 / MW_PI;
    bound2(gb, gl);
}

/* atSurveyGeometry.c:247-272 */
MWSEP_HD inline void gc_to_sgr(double mu, double nu, int wedge, double& lamda, double& beta)
{
    const double radpdeg = 3.141592653589793 / 180;
    mu = mu * radpdeg;
    nu = nu * radpdeg;
    const double x = cos(mu) * cos(nu);
    const double y = -sin(nu);
    const double z = sin(mu) * cos(nu);
    lamda = atan2(y, x);
    lamda = lamda / radpdeg;
    lamda = lamda + 2.5 * wedge;
    if (lamda < 0) lamda = lamda + 360;
    beta = asin(z);
    beta = beta / radpdeg;
}

/* The Sgr -> Galactic rotation: the Euler-angle matrix of phi=183.75,
 * theta=76.54, psi=194.111534 degrees (atSurveyGeometry.c:278-290), in its
 * reduced form.  The reference spells each entry as a ratio whose
 * denominator is identically one; sgr_rotation_ratio_form keeps that
 * spelling for host code that must round like the reference. */
MWSEP_HD inline void sgr_rotation(double* r)
{
    const double radpdeg = 3.141592653589793 / 180;
    const double phi = (180 + 3.75) * radpdeg;
    const double theta = (90 - 13.46) * radpdeg;
    const double psi = (180 + 14.111534) * radpdeg;
    const double cf = cos(phi), sf = sin(phi), ct = cos(theta), st = sin(theta), cp = cos(psi), sp = sin(psi);
    r[0] = cp * cf - ct * sf * sp;
    r[1] = -ct * sf * cp - sp * cf;
    r[2] = st * sf;
    r[3] = ct * cf * sp + cp * sf;
    r[4] = ct * cf * cp - sp * sf;
    r[5] = -st * cf;
    r[6] = sp * st;
    r[7] = cp * st;
    r[8] = ct;
}

/* Host only: the entries as the reference's ratios, with the terms formed
 * and summed in its order (same libm, same rounding). */
inline void sgr_rotation_ratio_form(double* r)
{
    const double radpdeg = 3.141592653589793 / 180;
    const double phi = (180 + 3.75) * radpdeg;
    const double theta = (90 - 13.46) * radpdeg;
    const double psi = (180 + 14.111534) * radpdeg;
    const double ct = cos(theta), st = sin(theta), cf = cos(phi), sf = sin(phi), cp = cos(psi), sp = sin(psi);
    const double ct2 = pow(ct, 2), st2 = pow(st, 2), cf2 = pow(cf, 2), sf2 = pow(sf, 2), cp2 = pow(cp, 2),
                 sp2 = pow(sp, 2);
    double d4 = cp2 * cf2 * ct2;
    d4 += cp2 * cf2 * st2;
    d4 += ct2 * sp2 * sf2;
    d4 += sp2 * cf2 * ct2;
    d4 += sp2 * cf2 * st2;
    d4 += ct2 * cp2 * sf2;
    d4 += st2 * sf2 * cp2;
    d4 += st2 * sf2 * sp2;
    const double d3a = ct2 * sf2 + cf2 * ct2 + cf2 * st2 + st2 * sf2;
    const double d3b = cp2 * ct2 + sp2 * st2 + cp2 * st2 + sp2 * ct2;
    r[0] = -(ct * sf * sp - ct2 * cf * cp - cp * st2 * cf) / d4;
    r[1] = -(ct * sf * cp + ct2 * cf * sp + sp * st2 * cf) / d4;
    r[2] = (st * sf) / d3a;
    r[3] = (ct * cf * sp + ct2 * cp * sf + cp * st2 * sf) / d4;
    r[4] = -(-ct * cf * cp + ct2 * sp * sf + sp * st2 * sf) / d4;
    r[5] = -(st * cf) / d3a;
    r[6] = (sp * st) / d3b;
    r[7] = (cp * st) / d3b;
    r[8] = ct / (ct2 + st2);
}

/* atSurveyGeometry.c:276-412: Sgr (lambda, beta) -> Galactic (l, b) with
 * the rotation rot (row-major). */
MWSEP_HD inline void sgr_to_gal(double lamda, double beta, const double* rot, double& l, double& b)
{
    const double radpdeg = 3.141592653589793 / 180;
    const double r11 = rot[0], r12 = rot[1], r13 = rot[2];
    const double r21 = rot[3], r22 = rot[4], r23 = rot[5];
    const double r31 = rot[6], r32 = rot[7], r33 = rot[8];
    double x2 = 0.0, y2 = 0.0;
    if (beta > 90)
    {
        beta = 90 - (beta - 90);
        lamda = lamda + 180;
        if (lamda > 360) lamda = lamda - 360;
    }
    if (beta < -90)
    {
        beta = -90 - (beta + 90);
        lamda = lamda + 180;
        if (lamda > 360) lamda = lamda - 360;
    }
    if (lamda < 0) lamda = lamda + 360;
    beta = beta + 90;
    beta = beta * radpdeg;
    const double z2 = cos(beta);
    if (lamda == 0) { x2 = sin(beta); y2 = 0; }
    else if (lamda < 90)
    {
        lamda = lamda * radpdeg;
        x2 = sqrt((1 - cos(beta) * cos(beta)) / (1 + tan(lamda) * tan(lamda)));
        y2 = x2 * tan(lamda);
    }
    else if (lamda == 90) { x2 = 0; y2 = sin(beta); }
    else if (lamda < 180)
    {
        lamda = lamda * radpdeg;
        y2 = sqrt((1 - cos(beta) * cos(beta)) / (1 / (tan(lamda) * tan(lamda)) + 1));
        x2 = y2 / tan(lamda);
    }
    else if (lamda == 180) { x2 = -sin(beta); y2 = 0; }
    else if (lamda < 270)
    {
        lamda = lamda * radpdeg;
        x2 = sqrt((1 - cos(beta) * cos(beta)) / (1 + tan(lamda) * tan(lamda)));
        y2 = x2 * tan(lamda);
        x2 = -x2;
        y2 = -y2;
    }
    else if (lamda == 270) { x2 = 0; y2 = -sin(beta); }
    else if (lamda < 360)
    {
        lamda = lamda * radpdeg;
        x2 = sqrt((1 - cos(beta) * cos(beta)) / (1 + tan(lamda) * tan(lamda)));
        y2 = x2 * tan(lamda);
    }
    else if (lamda == 360) { x2 = sin(beta); y2 = 0; }
    const double x1 = r11 * x2 + r12 * y2 + r13 * z2;
    const double y1 = r21 * x2 + r22 * y2 + r23 * z2;
    const double z1 = r31 * x2 + r32 * y2 + r33 * z2;
    if (z1 > 1) { l = 0; b = 90; }
    else
    {
        b = asin(z1);
        b = b / radpdeg;
        l = atan2(y1, x1);
        l = l / radpdeg;
        if (l < 0) l = l + 360;
    }
}

MWSEP_HD inline void sgr_to_gal(double lamda, double beta, double& l, double& b)
{
    double rot[9];
    sgr_rotation(rot);
    sgr_to_gal(lamda, beta, rot, l, b);
}

/* stCoords.c:108-130 */
MWSEP_HD inline double wedge_incl(int wedge)
{
    const double d = 2.5;
    return wedge * d - 57.5 - (wedge > 46 ? 180.0 : 0.0) + 32.5;
}


/* (mu, nu) of the wedge -> Galactic (l, b) in degrees:
 * cpu/evaluation_optimized.c:480-491 (cells) and :96-105 (stream centres). */
MWSEP_HD inline void wedge_point_lb(int sgr, int wedge, double mu, double nu, double& l, double& b)
{
    if (sgr == 0)
    {
        double ra, dec;
        gc_to_eq(mu, nu, 185.0 - 90.0, wedge_incl(wedge), ra, dec);
        eq_to_gal(ra, dec, l, b);
    }
    else
    {
        double lamda, beta;
        gc_to_sgr(mu, nu, wedge, lamda, beta);
        sgr_to_gal(lamda, beta, l, b);
    }
}

/* stCoords.c:33-48 (law of cosines, Sun at 8.5 kpc) */
MWSEP_HD inline void lbr_to_xyz(double l, double b, double r, double* xyz)
{
    const double r0 = 8.5;
    const double bsin = sin(b / MW_DEG), lsin = sin(l / MW_DEG);
    const double bcos = cos(b / MW_DEG), lcos = cos(l / MW_DEG);
    xyz[2] = r * bsin;
    const double zp = r * bcos;
    const double d = sqrt(r0 * r0 + zp * zp - 2 * r0 * zp * lcos);
    xyz[0] = (zp * zp - r0 * r0 - d * d) / (2 * r0);
    xyz[1] = zp * lsin;
}

/* set_probability_constants (cpu/evaluation_optimized.c:159-188) for one
 * distance `coords` (kpc): gPrime and reff_xr_rp3. */
MWSEP_HD inline void prob_consts_head(double coords, double& gPrime, double& reff_xr_rp3)
{
    gPrime = 5.0 * (log10(coords * 1000) - 1.0) + MW_ABSM;
    const double exp_result = exp(MW_SIG1 * (gPrime - MW_SIG2));
    const double reff_value = MW_SIG0 / (exp_result + 1);
    const double rPrime3 = coords * coords * coords;
    /* "xr" expands to 3 * stdev inside the product */
    reff_xr_rp3 = reff_value * 3 * MW_STDEV / rPrime3;
}

/* One convolution point of set_probability_constants: magnitude g,
 * r_point and qw_r3_N. */
MWSEP_HD inline void prob_consts_point(double gPrime, double dx, double gl_w, double coeff, double& g,
                                       double& r_point, double& qw_r3_N)
{
    g = gPrime + dx;
    r_point = pow(10.0, (g - MW_ABSM) / 5.0 + 1.0) / 1000.0;
    const double r3 = r_point * r_point * r_point;
    const double exponent = (g - gPrime) * (g - gPrime) / (2 * MW_STDEV * MW_STDEV);
    const double N = coeff * exp(-exponent);
    qw_r3_N = gl_w * r3 * N;
}

} // namespace mwsep

#endif
