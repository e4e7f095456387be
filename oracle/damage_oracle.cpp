// damage_oracle.cpp -- CPU restatement of AMIE's non-local Mazars damage step
// for StiffnessAndFracture on linear triangles (2D, plane stress).
//
// TEST INFRASTRUCTURE ONLY: the damage parity tests call it as the checker;
// the GPU library never links or loads it.
//
// What it restates (paths relative to the AMIE source tree):
//   geometry  Triangle::computeCenter (geometry/geometry_2D.cpp:507-515), the
//             circumradius of the Triangle constructor (:480-503), Triangle::area (:653-659)
//   caches    FractureCriterion::initialiseCache (physics/fracturecriteria/fracturecriterion.cpp:171-196)
//             through Mesh::generateCache (mesher/mesh.h:546-664), with the
//             QUARTIC_COMPACT smoothing function (fracturecriterion.cpp:46-52) and
//             the kernel size 2.5 (:29-31); membership by Circle::in (geometry/geometry_2D.cpp:1472-1484)
//   grade     FractureCriterion::step (fracturecriterion.cpp:534-560):
//             Mesh::getSmoothedFields (mesher/mesh.h:1384-1460, 1746-1790) of
//             PRINCIPAL_REAL_STRESS_FIELD and PRINCIPAL_TOTAL_STRAIN_FIELD,
//             toPrincipal (elements/integrable_entity.cpp:475-590) and
//             NonLocalMazars::gradeAtTime, 2D plane stress (physics/fracturecriteria/mazars.cpp:73-147)
//   update    FiberBasedIsotropicLinearDamage::step (physics/damagemodels/fiberbasedisotropiclineardamage.cpp:59-98),
//             FractureCriterion::getMaxScoreInNeighbourhood (fracturecriterion.cpp:251-280)
//
// The neighbour's strain enters the smoothing through ElementState::getAverageField
// with the cache weight (elements/integrable_entity.cpp:1992-2131): the
// one-point average (eps g c) / (g c), g the Gauss weight and c the cache
// weight, is set to zero when g c <= POINT_TOLERANCE, while the neighbour's
// a c still counts in the denominator (that happens at the edge of the kernel).
//
// Deviation, below the noise of the displacement solve: the cache order is
// element index order (the reference's is its Delaunay-tree order; only the
// rounding of the Kahan sums depends on it).
#include "amie_oracle.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

constexpr double kPointTolerance = 1e-12;   // POINT_TOLERANCE, geometry/geometry_base.h:292
constexpr double kKernelSize = 2.5;         // getSmoothingKernelSize, fracturecriterion.cpp:29-31

struct Circle {
    double cx, cy, r, r2;
    Circle(double x, double y, double radius) : cx(x), cy(y), r(radius), r2(radius * radius) {}
    bool in(double x, double y) const   // Circle::in
    {
        if (x < cx - r * 1.01 || x > cx + r * 1.01 || y < cy - r * 1.01 || y > cy + r * 1.01) return false;
        const double dx = x - cx, dy = y - cy;
        return dx * dx + dy * dy < r2;
    }
};

double reff(double R, double r) { return std::max(R, r * 1.1); }

// QUARTIC_COMPACT at (x, y) for a kernel centred on (cx, cy) with radius R:
// rrn = |p - c|^2 / R^2 / 2, (rrn - 1)^2 if 1 - rrn >= 0 else 0.
double quartic(double x, double y, double cx, double cy, double R)
{
    const double dx = x - cx, dy = y - cy;
    double rrn = (dx * dx + dy * dy) / (R * R);
    rrn = rrn / 2.;
    const double pos = (1. - rrn) >= 0 ? 1. : 0.;
    return (rrn - 1.) * (rrn - 1.) * pos;
}

// toPrincipal, 2D branch: SINGLE_OFF_DIAGONAL_VALUES (stress, v[2] = sxy) or
// DOUBLE_OFF_DIAGONAL_VALUES (strain, v[2] = engineering shear).
void principal(const double *v, bool engineering, double *out)
{
    const double trace = v[0] + v[1];
    const double det = engineering ? v[0] * v[1] - 0.25 * v[2] * v[2] : v[0] * v[1] - v[2] * v[2];
    const double delta = std::sqrt(trace * trace - 4. * det);
    const double angle = 0.5 * std::atan2(engineering ? 0.5 * v[2] : v[2], v[0] - v[1]);
    if (std::cos(angle) < 0) {
        out[0] = (trace + delta) * .5;
        out[1] = (trace - delta) * .5;
    } else {
        out[0] = (trace - delta) * .5;
        out[1] = (trace + delta) * .5;
    }
}

struct Mazars {   // NonLocalMazars(thresh, E, nu, Gf, radius, PLANE_STRESS): constants of its constructor
    double threshold, E, nu, B_t, B_c, A_c;
    explicit Mazars(const oracle_damage_law &l)
    {
        const double thresh = l.threshold, cstrain = -1., cstress = -1.;
        threshold = std::abs(thresh);
        E = l.young;
        nu = l.poisson;
        B_t = (0.1 * E * thresh) / (l.fracture_energy - E * 0.1 * thresh * thresh * 0.5);
        B_c = -1. / (std::sqrt(2.) * nu * cstrain);
        A_c = -(E * thresh + std::sqrt(2.) * cstress * nu) / ((E * std::exp(B_c * thresh - 1.) / B_c) - E * thresh);
    }
    // gradeAtTime for a 2D plane-stress element: principal smoothed stress and
    // strain, damage state of the element (its damage model's getState().max()).
    double grade(const double *stress, const double *strain, double dama_predict) const
    {
        const double strainzz = -nu * (strain[0] + strain[1]) / (1. - nu);
        double gamma = 1.0;
        const double Trtsig = 0.5 * (std::abs(stress[0]) + stress[0]) + 0.5 * (std::abs(stress[1]) + stress[1]);
        const double Trcsig = std::min(0.0, stress[0]) + std::min(0.0, stress[1]);
        if (Trcsig < -kPointTolerance && std::abs(Trtsig / Trcsig) < 1e-8)
            gamma = std::sqrt(std::min(0.0, stress[0]) * std::min(0.0, stress[0]) +
                              std::min(0.0, stress[1]) * std::min(0.0, stress[1])) / (-Trcsig);
        const double p0 = 0.5 * (std::abs(strain[0]) + strain[0]);
        const double p1 = 0.5 * (std::abs(strain[1]) + strain[1]);
        const double pz = 0.5 * (std::abs(strainzz) + strainzz);
        const double maxStrain = gamma * std::max(0.0, std::sqrt(p0 * p0 + p1 * p1 + pz * pz));
        // the 2D plane-stress branch sets tensionOnly, so talpha = 1 and calpha = 0
        const double talpha = 1.0, calpha = 1.0 - talpha;
        const double tt = std::max(threshold, maxStrain);
        const double pseudo = std::min(talpha * (1. - (threshold / tt) * (std::exp(-B_t * (tt - threshold)))) +
                                           calpha * (1. - (threshold * (1 - A_c) / tt) -
                                                     A_c * (std::exp(-B_c * (tt - threshold)))),
                                       1.0);
        return pseudo - dama_predict;
    }
};

}  // namespace

extern "C" int oracle_damage_geometry(uint32_t n, const double *xy, double *centre, double *radius, double *area)
{
    for (uint32_t e = 0; e < n; e++) {
        const double *p = xy + (size_t)e * 6;
        const double x0 = p[0], y0 = p[1], x1 = p[2], y1 = p[3], x2 = p[4], y2 = p[5];
        centre[2 * e] = ((0. + x0) + x1 + x2) / 3.;
        centre[2 * e + 1] = ((0. + y0) + y1 + y2) / 3.;
        // circumcentre (general position), radius as the mean distance of two vertices
        const double d = 2. * (x0 * (y1 - y2) + x1 * (y2 - y0) + x2 * (y0 - y1));
        const double s0 = x0 * x0 + y0 * y0, s1 = x1 * x1 + y1 * y1, s2 = x2 * x2 + y2 * y2;
        const double ux = (s0 * (y1 - y2) + s1 * (y2 - y0) + s2 * (y0 - y1)) / d;
        const double uy = (s0 * (x2 - x1) + s1 * (x0 - x2) + s2 * (x1 - x0)) / d;
        radius[e] = (std::hypot(x1 - ux, y1 - uy) + std::hypot(x0 - ux, y0 - uy)) / 2.;
        area[e] = 0.5 * std::abs((x0 - x1) * (y0 - y2) - (y0 - y1) * (x0 - x2));
    }
    return 0;
}

// Smoothing caches: for element e, every element whose centre is inside the
// circle of radius R_e 2.5 + 1.5 r_e (R_e = max(R, 1.1 r_e)) around e's centre,
// with the normalised weight mean_v max(w(v) a, 0) (w the kernel at the
// neighbour's three vertices, a its area).  idx == NULL: counts only (ptr).
extern "C" int oracle_damage_cache(uint32_t n, double R, const double *xy, const double *centre, const double *radius,
                                   const double *area, uint64_t *ptr, uint32_t *idx, double *coef)
{
    ptr[0] = 0;
    std::vector<uint32_t> members;
    std::vector<double> w;
    for (uint32_t e = 0; e < n; e++) {
        const double Re = reff(R, radius[e]);
        const Circle c(centre[2 * e], centre[2 * e + 1], Re * kKernelSize + radius[e] * 1.5);
        members.clear();
        w.clear();
        for (uint32_t j = 0; j < n; j++) {
            if (!c.in(centre[2 * j], centre[2 * j + 1])) continue;
            double k = 0;
            for (int v = 0; v < 3; v++)
                k += std::max(quartic(xy[(size_t)j * 6 + 2 * v], xy[(size_t)j * 6 + 2 * v + 1], c.cx, c.cy, Re) *
                                  area[j], 0.);
            k /= 3;
            if (k < kPointTolerance * kPointTolerance) continue;
            members.push_back(j);
            w.push_back(k);
        }
        double tot = 0;
        for (double x : w) tot += x;
        ptr[e + 1] = ptr[e] + members.size();
        if (idx)
            for (size_t k = 0; k < members.size(); k++) {
                idx[ptr[e] + k] = members[k];
                coef[ptr[e] + k] = w[k] / tot;
            }
    }
    return 0;
}

extern "C" int oracle_damage_grade(uint32_t n, const oracle_damage_law *law, const double *strain,
                                   const double *cmat, const double *state, const double *area, const double *gpw,
                                   const uint64_t *ptr, const uint32_t *idx, const double *coef, double *score,
                                   double *smoothed)
{
    const Mazars mz(*law);
    auto fractured = [&](uint32_t e) { return state[e] >= law->cutoff; };
    for (uint32_t e = 0; e < n; e++) {
        double sc[3] = {0, 0, 0}, corr[3] = {0, 0, 0}, sum = 0;
        for (uint64_t k = ptr[e]; k < ptr[e + 1]; k++) {
            const uint32_t j = idx[k];
            if (fractured(j)) continue;
            const double v = area[j] * coef[k];
            const double tot = gpw[j] * coef[k];
            for (int c = 0; c < 3; c++) {
                const double avg = tot > kPointTolerance ? strain[(size_t)j * 3 + c] * gpw[j] * coef[k] / tot : 0.;
                const double y = avg * v - corr[c];
                const double t = sc[c] + y;
                corr[c] = (t - sc[c]) - y;
                sc[c] = t;
            }
            sum += v;
        }
        for (int c = 0; c < 3; c++) sc[c] = sum > kPointTolerance ? sc[c] / sum : 0.;
        const double f = fractured(e) ? law->residual : 1. - state[e];
        const double *C = cmat + (size_t)e * 9;
        double sig[3];
        const double g = gpw[e];
        for (int i = 0; i < 3; i++) {   // Vector * Matrix: column i of C_eff against the strain
            double s = 0;
            for (int k = 0; k < 3; k++) s = s + (C[k * 3 + i] * f) * sc[k];
            sig[i] = g > kPointTolerance * kPointTolerance ? s * g / g : s * g;   // one-point average
        }
        double ps[2], pe[2];
        principal(sig, false, ps);
        principal(sc, true, pe);
        if (smoothed) {
            smoothed[4 * e] = ps[0];
            smoothed[4 * e + 1] = ps[1];
            smoothed[4 * e + 2] = pe[0];
            smoothed[4 * e + 3] = pe[1];
        }
        score[e] = fractured(e) ? -1. : mz.grade(ps, pe, state[e]);
    }
    return 0;
}

extern "C" int oracle_damage_update(uint32_t n, const oracle_damage_law *law, const double *centre,
                                    const double *radius, const double *score, double *state, uint8_t *changed)
{
    // Elements are stepped one after the other in mesh order (the order of
    // FeatureTree::stepElements' loop, features/features.cpp:5062-5088, with one
    // thread): an element that becomes fractured leaves the neighbourhood
    // maxima of the elements stepped after it.
    std::vector<uint8_t> fr(n);
    for (uint32_t e = 0; e < n; e++) fr[e] = state[e] >= law->cutoff;
    for (uint32_t e = 0; e < n; e++) {
        changed[e] = 0;
        if (!(score[e] > 0)) continue;   // criterion not met
        const double Re = reff(law->radius, radius[e]);
        const Circle all(centre[2 * e], centre[2 * e + 1], std::max(Re * 6., radius[e] * 4.) * kKernelSize + radius[e]);
        double nmax = score[e];
        for (uint32_t j = 0; j < n; j++)
            if (!fr[j] && all.in(centre[2 * j], centre[2 * j + 1])) nmax = std::max(nmax, score[j]);
        if (!fr[e] && std::abs(score[e] - nmax) < law->score_tolerance) {
            state[e] += law->fibre;
            if (state[e] > 1) state[e] = 1;
            changed[e] = 1;
            fr[e] = state[e] >= law->cutoff;
        }
    }
    return 0;
}
