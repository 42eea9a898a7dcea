// Gauss-linear-corrected Laplacian of a tensor conductivity on a general
// mesh, assembled on the host once per context (the conductivity is static).
//
// Per internal face f (owner P, neighbour N, area vector Sf from P to N):
//   weight       w   = |Sf.(C_N - Cf)| / (|Sf.(Cf - C_P)| + |Sf.(C_N - Cf)|)
//   deltaCoeff   dc  = 1 / max(n.d, 0.05 |d|),  n = Sf/|Sf|, d = C_N - C_P
//   corrVec          = n - dc d
//   Gamma_f          = w (Gamma_P - Gamma_N) + Gamma_N
//   SfGamma          = Sf . Gamma_f,  SfGammaSn = SfGamma . n,
//   SfGammaCorr      = SfGamma - SfGammaSn n
//   upper()          = dc SfGammaSn                           (implicit)
//   correction flux  = SfGammaCorr.g_f + SfGammaSn corrVec.g_f  (explicit)
// with g_f = w (g_P - g_N) + g_N the cell gradient interpolated to the face.
// Wall faces (zeroGradient Vm, the wall's conductivity the cell's) add
// SfGammaCorr.(g_P - n (n.g_P)) to their cell.  The cell gradient is
// leastSquares (vectors invDd.d/|d|^2 with dd the sum of d d/|d|^2 over the
// cell's faces, walls using the patch-normal delta n (n.(Cf - C))) or Gauss
// linear (face values by linear interpolation, divided by the volume).
// Both gradients are stored as weights of neighbour differences: a row's
// gradient is sum_e gw_e (phi_nb - phi_c); for Gauss linear this drops
// phi_c times the cell's closed-surface sum of Sf, which is zero up to
// round-off.
#include "geometry.h"

#include <cmath>

#include "host_common.h"

namespace cfg {

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 load(const double* p, long long i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
inline void store(double* p, long long i, V3 v)
{
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

// full tensor (row-major) of a symmTensor xx xy xz yy yz zz
inline void full(const double* s, double t[9])
{
    t[0] = s[0]; t[1] = s[1]; t[2] = s[2];
    t[3] = s[1]; t[4] = s[3]; t[5] = s[4];
    t[6] = s[2]; t[7] = s[4]; t[8] = s[5];
}

// Sf . Gamma (row vector times tensor)
inline V3 vdott(V3 S, const double* G)
{
    return {S.x * G[0] + S.y * G[3] + S.z * G[6], S.x * G[1] + S.y * G[4] + S.z * G[7],
            S.x * G[2] + S.y * G[5] + S.z * G[8]};
}

// SfGammaSn and SfGammaCorr of one face
inline double face_gamma(V3 S, const double* G, V3& corr)
{
    const double mag = std::sqrt(dot(S, S));
    const V3 n{S.x / mag, S.y / mag, S.z / mag};
    const V3 sg = vdott(S, G);
    const double sn = dot(sg, n);
    corr = sg - sn * n;
    return sn;
}

}  // namespace

int assemble_corrected(const cfg_mesh_desc* m, const double* sigma_uniform,
                       const double* sigma_cells, int grad_scheme, int uncorrected,
                       CorrectedOperator& op)
{
    const long long n = m->n_cells, nf = m->n_faces, nb = m->n_boundary_faces;
    if (!m->face_centres || !m->face_sf || !m->centres || !m->volumes)
        return fail(CFG_ERR_INVALID, "a general mesh needs face_centres, face_sf, centres and volumes");
    if (nb < 0 || (nb > 0 && (!m->boundary_cell || !m->boundary_sf || !m->boundary_centres)))
        return fail(CFG_ERR_INVALID, "boundary faces need boundary_cell, boundary_sf and boundary_centres");
    if (grad_scheme != CFG_GRAD_LEAST_SQUARES && grad_scheme != CFG_GRAD_GAUSS_LINEAR)
        return fail(CFG_ERR_INVALID, "unknown gradient scheme %d", grad_scheme);
    for (long long b = 0; b < nb; ++b)
        if (m->boundary_cell[b] < 0 || m->boundary_cell[b] >= n)
            return fail(CFG_ERR_INVALID, "boundary face %lld has invalid cell %d", b,
                        m->boundary_cell[b]);
    const double* C = m->centres;
    const double* V = m->volumes;
    auto sigma = [&](long long c, double t[9]) {
        full(sigma_cells ? sigma_cells + 6 * c : sigma_uniform, t);
    };
    op.coeff.assign(size_t(nf), 0.0);
    op.w.assign(size_t(nf), 0.0);
    op.k.assign(size_t(3 * nf), 0.0);
    op.g_own.assign(size_t(3 * nf), 0.0);
    op.g_nei.assign(size_t(3 * nf), 0.0);
    op.bk.assign(size_t(3 * n), 0.0);
    std::vector<double> dd(size_t(6 * n), 0.0);
    auto add_dd = [&](long long c, V3 d) {
        const double m2 = dot(d, d);
        double* a = dd.data() + 6 * c;
        a[0] += d.x * d.x / m2; a[1] += d.x * d.y / m2; a[2] += d.x * d.z / m2;
        a[3] += d.y * d.y / m2; a[4] += d.y * d.z / m2; a[5] += d.z * d.z / m2;
    };
    for (long long f = 0; f < nf; ++f) {
        const long long P = m->owner[f], N = m->neighbour[f];
        const V3 S = load(m->face_sf, f), Cf = load(m->face_centres, f);
        const V3 CP = load(C, P), CN = load(C, N);
        const double mag = std::sqrt(dot(S, S));
        if (!(mag > 0.0)) return fail(CFG_ERR_INVALID, "face %lld has zero area", f);
        const V3 nrm{S.x / mag, S.y / mag, S.z / mag};
        const double own = std::fabs(dot(S, Cf - CP)), nei = std::fabs(dot(S, CN - Cf));
        const double w = nei / (own + nei);
        const V3 d = CN - CP;
        const double md = std::sqrt(dot(d, d));
        const double nd = dot(nrm, d);
        const double dc = 1.0 / (nd > 0.05 * md ? nd : 0.05 * md);
        const V3 corr_vec = nrm - dc * d;
        double GP[9], GN[9], G[9];
        sigma(P, GP);
        sigma(N, GN);
        for (int q = 0; q < 9; ++q) G[q] = w * (GP[q] - GN[q]) + GN[q];
        V3 sgc;
        const double sgsn = face_gamma(S, G, sgc);
        op.coeff[size_t(f)] = dc * sgsn;
        op.w[size_t(f)] = w;
        store(op.k.data(), f, uncorrected ? sgc : sgc + sgsn * corr_vec);
        if (grad_scheme == CFG_GRAD_LEAST_SQUARES) {
            add_dd(P, d);
            add_dd(N, d);
        } else {
            store(op.g_own.data(), f, ((1.0 - w) / V[P]) * S);
            store(op.g_nei.data(), f, (-w / V[N]) * S);
        }
    }
    for (long long b = 0; b < nb; ++b) {
        const long long P = m->boundary_cell[b];
        const V3 S = load(m->boundary_sf, b);
        const double mag = std::sqrt(dot(S, S));
        if (!(mag > 0.0)) return fail(CFG_ERR_INVALID, "boundary face %lld has zero area", b);
        const V3 nrm{S.x / mag, S.y / mag, S.z / mag};
        double G[9];
        sigma(P, G);
        V3 sgc;
        (void)face_gamma(S, G, sgc);
        const V3 wall = sgc - dot(sgc, nrm) * nrm;
        store(op.bk.data(), P, load(op.bk.data(), P) + wall);
        if (grad_scheme == CFG_GRAD_LEAST_SQUARES) {
            const V3 r = load(m->boundary_centres, b) - load(C, P);
            add_dd(P, dot(nrm, r) * nrm);
        }
    }
    if (grad_scheme == CFG_GRAD_LEAST_SQUARES) {
        for (long long c = 0; c < n; ++c) {
            double* a = dd.data() + 6 * c;
            const double xx = a[0], xy = a[1], xz = a[2], yy = a[3], yz = a[4], zz = a[5];
            const double det = xx * (yy * zz - yz * yz) - xy * (xy * zz - xz * yz) +
                               xz * (xy * yz - yy * xz);
            if (!(std::fabs(det) > 0.0))
                return fail(CFG_ERR_INVALID, "cell %lld: singular least-squares matrix", c);
            a[0] = (yy * zz - yz * yz) / det;
            a[1] = (xz * yz - xy * zz) / det;
            a[2] = (xy * yz - xz * yy) / det;
            a[3] = (xx * zz - xz * xz) / det;
            a[4] = (xy * xz - xx * yz) / det;
            a[5] = (xx * yy - xy * xy) / det;
        }
        auto mul = [&](long long c, V3 d) {
            const double* a = dd.data() + 6 * c;
            return V3{a[0] * d.x + a[1] * d.y + a[2] * d.z, a[1] * d.x + a[3] * d.y + a[4] * d.z,
                      a[2] * d.x + a[4] * d.y + a[5] * d.z};
        };
        for (long long f = 0; f < nf; ++f) {
            const long long P = m->owner[f], N = m->neighbour[f];
            const V3 d = load(C, N) - load(C, P);
            const double k = 1.0 / dot(d, d);
            // leastSquaresGrad: g_P += k invDd_P.d (phi_N - phi_P) and
            // g_N -= (-k invDd_N.d) (phi_N - phi_P), so the neighbour's weight
            // of its own difference (phi_P - phi_N) is -k invDd_N.d
            store(op.g_own.data(), f, k * mul(P, d));
            store(op.g_nei.data(), f, (-k) * mul(N, d));
        }
    }
    return CFG_OK;
}

}  // namespace cfg
