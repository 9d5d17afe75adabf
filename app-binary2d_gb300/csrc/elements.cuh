// elements.cuh — change of the binary's orbital elements under a block's
// accreted mass and momentum.
//
// ItemizedChange::perturbation (src/state.rs:258-281) calls
// OrbitalElements::perturb of kepler-two-body (un-vendored; restated here
// from two-body mechanics): at the stage time, body k gains mass dm_k and
// momentum dp_k at fixed position; the perturbed elements (a, M, q, e) follow
// from the new relative orbit — M' = m1' + m2', q' = m2'/m1', specific energy
// E = |v|²/2 - M'/|r| gives a' = -M'/(2E), angular momentum h = r × v gives
// e' = sqrt(1 + 2 E h² / M'²).  An orbit with E >= 0 is unbound
// (UnboundOrbitalState, physics.rs:34-35).
#pragma once

namespace b2d {

// orbit: m, x, y, vx, vy of body 1 then body 2 at the stage time; el: the
// unperturbed (a, M, q, e).  Writes perturbed - unperturbed into de; returns
// false when the perturbed orbit is unbound.
__host__ __device__ inline bool perturb_elements(const double* orbit, const double* el, double dm1, double dm2,
                                                 double dpx1, double dpx2, double dpy1, double dpy2, double* de)
{
    const double m1 = orbit[0], x1 = orbit[1], y1 = orbit[2], vx1 = orbit[3], vy1 = orbit[4];
    const double m2 = orbit[5], x2 = orbit[6], y2 = orbit[7], vx2 = orbit[8], vy2 = orbit[9];
    const double m1n = m1 + dm1, m2n = m2 + dm2;
    const double ux1 = (m1 * vx1 + dpx1) / m1n, uy1 = (m1 * vy1 + dpy1) / m1n;
    const double ux2 = (m2 * vx2 + dpx2) / m2n, uy2 = (m2 * vy2 + dpy2) / m2n;
    const double M = m1n + m2n, q = m2n / m1n;
    const double rx = x2 - x1, ry = y2 - y1, vx = ux2 - ux1, vy = uy2 - uy1;
    const double r = sqrt(rx * rx + ry * ry);
    const double E = 0.5 * (vx * vx + vy * vy) - M / r;
    if (!(E < 0.0)) return false;
    const double a = -M / (2.0 * E);
    const double h = rx * vy - ry * vx;
    const double ee = 1.0 + 2.0 * E * h * h / (M * M);
    const double e = ee > 0.0 ? sqrt(ee) : 0.0;
    de[0] = a - el[0];
    de[1] = M - el[1];
    de[2] = q - el[2];
    de[3] = e - el[3];
    return true;
}

}  // namespace b2d
