// Body, gravitational and centrifugal loads: the body-force branch of getElasticAppliedLoad
// (Working/AStrO_commandFunctions.f90:393-441) with r_getElBodyForce
// (Working/AStrO_r_elementEqns.f90:1801-1869) and r_getElCentAcc (:1871-1921).
//   bricks: one thread per listed element, launched colour by colour (no two elements of a colour
//           share a node, so the additions need no atomics and have a fixed order); the nodal
//           forces are b or rho a (the brick's consistent mass times a uniform acceleration)
//           times the integral of N over the element;
//   shells: body force: one thread per element, t b times the integral of N over the element in
//           its frame (all six nodal components); gravitational and centrifugal loads: the
//           element mass residual for the acceleration (r_getElRum with the static frame of the
//           element's mean rotation), which the shell pipeline evaluates as the Newmark mass term:
//           run alone (massOnly) with a previous-acceleration field that makes the Newmark
//           acceleration the imposed one.  The centrifugal acceleration differs per element; it
//           goes into the field at the element's nodes one colour at a time (a colour's elements
//           share no node).  An element listed k times is evaluated in k passes.
#include <algorithm>
#include <cmath>
#include <functional>
#include <string>
#include <vector>

#include "astro_internal.h"
#include "shell_props.cuh"

namespace {

struct BodyVals {
    double v[7];
};

// one listed brick element of a colour per thread
__global__ void k_hex_body(int kind, BodyVals bv, const int *__restrict__ els, int cnt, const double *__restrict__ nodes,
                           const int *__restrict__ elist, const int *__restrict__ rank, const double *__restrict__ disp,
                           const double *__restrict__ den, const double *__restrict__ mult,
                           double *__restrict__ load) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    const int e = els[i];
    double X[8][3];
    int r[8];
    for (int k = 0; k < 8; ++k) {
        const int nd = elist[8 * (size_t)e + k] - 1;
        r[k] = rank[nd] - 1;
        for (int d = 0; d < 3; ++d) X[k][d] = nodes[3 * (size_t)nd + d];
    }
    double a[3];
    if (kind == 2) {
        // r_getElCentAcc: omega^2 times the centroid's distance vector from the axis
        double c[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 8; ++k)
            for (int d = 0; d < 3; ++d) c[d] = c[d] + X[k][d] + (disp ? disp[3 * (size_t)r[k] + d] : 0.0);
        const double nnInv = 1.0 / 8.0;
        double pos[3], unit[3];
        for (int d = 0; d < 3; ++d) pos[d] = nnInv * c[d] - bv.v[d];
        double dp = bv.v[3] * bv.v[3] + bv.v[4] * bv.v[4] + bv.v[5] * bv.v[5];
        const double mag = sqrt(dp);
        for (int d = 0; d < 3; ++d) unit[d] = (1.0 / mag) * bv.v[3 + d];
        dp = pos[0] * unit[0] + pos[1] * unit[1] + pos[2] * unit[2];
        for (int d = 0; d < 3; ++d) a[d] = bv.v[6] * bv.v[6] * (pos[d] - dp * unit[d]);
    } else {
        for (int d = 0; d < 3; ++d) a[d] = bv.v[d];
    }
    const double f = ((kind >= 1) ? den[e] : 1.0) * mult[i];
    // integral of N_k over the element, 2 x 2 x 2 Gauss points at +-1/sqrt(3)
    const double g = 1.0 / sqrt(3.0);
    const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                 sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int gp = 0; gp < 8; ++gp) {
        const double s1 = g * sx[gp], s2 = g * sy[gp], s3 = g * sz[gp];
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, N[8];
        for (int k = 0; k < 8; ++k) {
            const double a1 = 1.0 + sx[k] * s1, a2 = 1.0 + sy[k] * s2, a3 = 1.0 + sz[k] * s3;
            N[k] = 0.125 * a1 * a2 * a3;
            const double d1 = 0.125 * sx[k] * a2 * a3, d2 = 0.125 * sy[k] * a1 * a3, d3 = 0.125 * sz[k] * a1 * a2;
            for (int d = 0; d < 3; ++d) {
                J[d][0] += X[k][d] * d1;
                J[d][1] += X[k][d] * d2;
                J[d][2] += X[k][d] * d3;
            }
        }
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        for (int k = 0; k < 8; ++k) w[k] += N[k] * det;
    }
    for (int k = 0; k < 8; ++k)
        for (int d = 0; d < 3; ++d) load[3 * (size_t)r[k] + d] += f * a[d] * w[k];
}

// out += s a
__global__ void k_add_scaled(int n, double s, const double *__restrict__ a, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += s * a[i];
}

// out -= b (the pipeline's output is the load -Ru)
// centripetal acceleration omega^2 (pos - (pos . axis) axis) at centroid c (r_getElCentAcc)
__device__ __forceinline__ void cent_acc(const BodyVals &bv, const double c[3], double a[3]) {
    double pos[3], unit[3];
    for (int d = 0; d < 3; ++d) pos[d] = c[d] - bv.v[d];
    double dp = bv.v[3] * bv.v[3] + bv.v[4] * bv.v[4] + bv.v[5] * bv.v[5];
    const double mag = sqrt(dp);
    for (int d = 0; d < 3; ++d) unit[d] = (1.0 / mag) * bv.v[3 + d];
    dp = pos[0] * unit[0] + pos[1] * unit[1] + pos[2] * unit[2];
    for (int d = 0; d < 3; ++d) a[d] = bv.v[6] * bv.v[6] * (pos[d] - dp * unit[d]);
}

// shell body force: t b_c times the integral of N_a over the element (frame of its properties)
__global__ void k_shell_body(BodyVals bv, const int *__restrict__ els, int cnt, const double *__restrict__ nodes,
                             const int *__restrict__ elist, const int *__restrict__ rank,
                             const ShellProps *__restrict__ props, const int *__restrict__ esec,
                             const int *__restrict__ layRange, const LayerDev *__restrict__ lay,
                             const int *__restrict__ e2dR, const int *__restrict__ e2d, const double *__restrict__ e2c,
                             const int *__restrict__ dcat, const int *__restrict__ dlay, const double *__restrict__ dval,
                             const double *__restrict__ mult, const double *__restrict__ tOverride,
                             double *__restrict__ load) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    const int e = els[i];
    double Xl[4][3];
    int r[4];
    for (int a = 0; a < 4; ++a) {
        const int nd = elist[8 * (size_t)e + a] - 1;
        r[a] = rank[nd] - 1;
        for (int k = 0; k < 3; ++k) {
            double s = 0.0;
            for (int j = 0; j < 3; ++j) s += props[e].orient[3 * k + j] * nodes[3 * (size_t)nd + j];
            Xl[a][k] = s;
        }
    }
    // section thickness with the layer-thickness design variables (or the given per-element factor)
    const int sec = esec[e];
    double t = 0.0;
    if (tOverride) t = tOverride[e];
    for (int li = layRange[sec - 1], ln = 1; !tOverride && li < layRange[sec]; ++li, ++ln) {
        double tl = lay[li].t;
        if (e2dR)
            for (int q = e2dR[e]; q < e2dR[e + 1]; ++q) {
                const int d = e2d[q] - 1;
                if (dcat[d] == ASTRO_DCAT_LAYUP_THICKNESS && dlay[d] == ln) tl = tl + e2c[q] * dval[d];
            }
        t = t + tl;
    }
    const double g = 1.0 / sqrt(3.0);
    const double sx[4] = {-1.0, 1.0, 1.0, -1.0}, sy[4] = {-1.0, -1.0, 1.0, 1.0};
    double w[4] = {0.0, 0.0, 0.0, 0.0};
    for (int gp = 0; gp < 4; ++gp) {
        const double s1 = (gp & 1) ? g : -g, s2 = (gp & 2) ? g : -g;
        double J[2][2] = {{0.0, 0.0}, {0.0, 0.0}}, N[4];
        for (int a = 0; a < 4; ++a) {
            N[a] = 0.25 * (1.0 + sx[a] * s1) * (1.0 + sy[a] * s2);
            const double d0 = 0.25 * sx[a] * (1.0 + sy[a] * s2), d1 = 0.25 * sy[a] * (1.0 + sx[a] * s1);
            for (int k = 0; k < 2; ++k) {
                J[k][0] += Xl[a][k] * d0;
                J[k][1] += Xl[a][k] * d1;
            }
        }
        // dxds(3,3) = 1 and no thickness-direction parameter: det = J00 J11 - J01 J10
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        for (int a = 0; a < 4; ++a) w[a] += N[a] * det;
    }
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 6; ++c) load[6 * (size_t)r[a] + c] += mult[i] * (t * (bv.v[c] * w[a]));
}

// centrifugal acceleration of each listed element (displaced centroid) into the previous-
// acceleration field at its nodes, negated (the Newmark acceleration then equals it)
__global__ void k_shell_cent_pacc(BodyVals bv, const int *__restrict__ els, int cnt, const double *__restrict__ nodes,
                                  const int *__restrict__ elist, const int *__restrict__ rank,
                                  const double *__restrict__ disp, double *__restrict__ pacc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    const int e = els[i];
    int r[4];
    double c[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < 4; ++a) {
        const int nd = elist[8 * (size_t)e + a] - 1;
        r[a] = rank[nd] - 1;
        for (int d = 0; d < 3; ++d) c[d] = c[d] + nodes[3 * (size_t)nd + d] + (disp ? disp[6 * (size_t)r[a] + d] : 0.0);
    }
    const double nnInv = 1.0 / 4.0;
    for (int d = 0; d < 3; ++d) c[d] = nnInv * c[d];
    double acc[3];
    cent_acc(bv, c, acc);
    for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 6; ++d) pacc[6 * (size_t)r[a] + d] = d < 3 ? -acc[d] : 0.0;
}

__global__ void k_sub(int n, const double *__restrict__ b, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] -= b[i];
}

}  // namespace

extern "C" int astro_body_load(astro_ctx *ctx, int32_t kind, const double *vals, const int32_t *elements, int32_t count,
                               const astro_state *state, double *elastic_load) {
    if (!ctx || !vals || !elastic_load || kind < 0 || kind > 2 || count < 0) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    const int n = P.n;
    if (ctx->hasShell && ctx->hasSolid) return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "body loads on mixed meshes");
    if (elements)
        for (int k = 0; k < count; ++k)
            if (elements[k] < 1 || elements[k] > P.E) return set_err(ctx, ASTRO_ERR_ARG, "element number out of range");
    if (elements && count == 0) return ASTRO_OK;
    struct Tmp {
        DevBuf ref, li, u, b, list, mult, den, pa, iu;
        ~Tmp() {
            DevBuf *v[] = {&ref, &li, &u, &b, &list, &mult, &den, &pa, &iu};
            for (DevBuf *p : v) dev_free(*p);
        }
    } T;
    int rc;
    if ((rc = dev_alloc(ctx, T.ref, sizeof(double) * n)) || (rc = dev_alloc(ctx, T.li, sizeof(double) * n))) return rc;
    CK(cudaMemcpyAsync(T.ref.p, elastic_load, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = ref_to_int_vec(ctx, dptr<double>(T.ref), dptr<double>(T.li), n))) return rc;
    if (state && state->node_disp) {
        DevBuf h;
        rc = upload(ctx, h, state->node_disp, sizeof(double) * n);
        if (!rc) rc = dev_alloc(ctx, T.u, sizeof(double) * n);
        if (!rc) rc = ref_to_int_vec(ctx, dptr<double>(h), dptr<double>(T.u), n);
        if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "state upload");
        dev_free(h);
        if (rc) return rc;
    }
    // the listed elements, colour by colour, with their multiplicity (an element listed twice
    // adds its load twice)
    std::vector<int> on((size_t)P.E, elements ? 0 : 1);
    if (elements)
        for (int k = 0; k < count; ++k) ++on[elements[k] - 1];
    BodyVals bv;
    for (int k = 0; k < 7; ++k) bv.v[k] = (kind == 2 || k < 6) ? vals[k] : 0.0;
    if (ctx->hasSolid || kind == 0) {
        std::vector<int> list, ptr(1, 0);
        std::vector<double> mult;
        for (int col = 0; col < P.ncolors; ++col) {
            for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k)
                if (on[P.colorEls[k]]) {
                    list.push_back(P.colorEls[k]);
                    mult.push_back((double)on[P.colorEls[k]]);
                }
            ptr.push_back((int)list.size());
        }
        if (!list.empty()) {
            if ((rc = upload(ctx, T.list, list.data(), sizeof(int) * list.size())) ||
                (rc = upload(ctx, T.mult, mult.data(), sizeof(double) * mult.size())))
                return rc;
            if (ctx->hasSolid &&
                (rc = upload(ctx, T.den, ctx->elDensity.data(), sizeof(double) * ctx->elDensity.size())))
                return rc;
            const bool dv = ctx->numDvars > 0 && ctx->d_e2dR.p;
            for (int col = 0; col < P.ncolors; ++col) {
                const int cnt = ptr[col + 1] - ptr[col];
                if (!cnt) continue;
                if (ctx->hasSolid)
                    k_hex_body<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(
                        kind, bv, dptr<int>(T.list) + ptr[col], cnt, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist),
                        dptr<int>(ctx->d_rank), T.u.p ? dptr<double>(T.u) : nullptr, dptr<double>(T.den),
                        dptr<double>(T.mult) + ptr[col], dptr<double>(T.li));
                else
                    k_shell_body<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(
                        bv, dptr<int>(T.list) + ptr[col], cnt, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist),
                        dptr<int>(ctx->d_rank), dptr<ShellProps>(ctx->d_secABD), dptr<int>(ctx->d_esec),
                        dptr<int>(ctx->d_shLayRange), dptr<LayerDev>(ctx->d_shLay), dv ? dptr<int>(ctx->d_e2dR) : nullptr,
                        dv ? dptr<int>(ctx->d_e2d) : nullptr, dv ? dptr<double>(ctx->d_e2c) : nullptr,
                        dv ? dptr<int>(ctx->d_dCat) : nullptr, dv ? dptr<int>(ctx->d_dLayer) : nullptr,
                        dv ? dptr<double>(ctx->d_dVal) : nullptr, dptr<double>(T.mult) + ptr[col], nullptr,
                        dptr<double>(T.li));
            }
            if ((rc = cuda_check(ctx, cudaGetLastError(), "body load"))) return rc;
        }
    } else {
        // shells, gravitational / centrifugal: load += Rum, the Newmark mass residual alone (the
        // elastic part is left out, not subtracted: at a displaced state it is orders of
        // magnitude larger)
        const bool zeroState = !T.u.p;
        if (zeroState) {
            if ((rc = dev_alloc(ctx, T.u, sizeof(double) * n))) return rc;
            CK(cudaMemsetAsync(T.u.p, 0, sizeof(double) * n, ctx->stream));
        }
        const int ni = P.intVecSize;
        if (ni > 0) {
            if (state && state->internal_disp) {
                if ((rc = upload(ctx, T.iu, state->internal_disp, sizeof(double) * ni))) return rc;
            } else {
                if ((rc = dev_alloc(ctx, T.iu, sizeof(double) * ni))) return rc;
                CK(cudaMemsetAsync(T.iu.p, 0, sizeof(double) * ni, ctx->stream));
            }
        }
        // previous acceleration -a at the nodes: with u = u_prev, v_prev = 0 and beta = 1/4 the
        // Newmark acceleration is a
        std::vector<double> pa((size_t)n, 0.0);
        if (kind == 1)
            for (int r = 0; r < P.N; ++r)
                for (int c = 0; c < P.dpn; ++c) pa[(size_t)r * P.dpn + c] = -vals[c];
        if ((rc = upload(ctx, T.pa, pa.data(), sizeof(double) * n))) return rc;
        if ((rc = dev_alloc(ctx, T.b, sizeof(double) * n))) return rc;
        CK(cudaMemsetAsync(T.b.p, 0, sizeof(double) * n, ctx->stream));
        ElemDevState s1;
        s1.disp = dptr<double>(T.u);
        s1.idisp = ni > 0 ? dptr<double>(T.iu) : nullptr;
        s1.pdisp = s1.disp;
        s1.pacc = dptr<double>(T.pa);
        s1.pidisp = s1.idisp;
        s1.dynamic = 1;
        s1.beta = 0.25;
        s1.gamma = 0.5;
        s1.delT = 1.0;
        s1.massOnly = 1;
        const int maxMult = *std::max_element(on.begin(), on.end());
        for (int pass = 0; pass < maxMult; ++pass) {
            std::vector<int> list, ptr(1, 0);
            for (int col = 0; col < P.ncolors; ++col) {
                for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k)
                    if (on[P.colorEls[k]] > pass) list.push_back(P.colorEls[k]);
                ptr.push_back((int)list.size());
            }
            if (list.empty()) continue;
            dev_free(T.list);
            if ((rc = upload(ctx, T.list, list.data(), sizeof(int) * list.size()))) return rc;
            if (kind == 1) {
                if ((rc = shell4_residual_list(ctx, s1, dptr<int>(T.list), ptr, dptr<double>(T.b)))) return rc;
                continue;
            }
            for (int col = 0; col < P.ncolors; ++col) {
                const int cnt = ptr[col + 1] - ptr[col];
                if (!cnt) continue;
                k_shell_cent_pacc<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(
                    bv, dptr<int>(T.list) + ptr[col], cnt, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist),
                    dptr<int>(ctx->d_rank), zeroState ? nullptr : dptr<double>(T.u), dptr<double>(T.pa));
                const std::vector<int> one = {ptr[col], ptr[col + 1]};
                if ((rc = shell4_residual_list(ctx, s1, dptr<int>(T.list), one, dptr<double>(T.b)))) return rc;
            }
        }
        k_sub<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, dptr<double>(T.b), dptr<double>(T.li));
        if ((rc = cuda_check(ctx, cudaGetLastError(), "shell mass load"))) return rc;
    }
    if ((rc = int_to_ref_vec(ctx, dptr<double>(T.li), dptr<double>(T.ref), n))) return rc;
    CK(cudaMemcpyAsync(elastic_load, T.ref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

// d(body load)/d(design variable): drudd -= dF/dd for the listed elements that depend on dvar,
// the load branch of getdRelasticdD (Working/AStrO_commandFunctions.f90:1250-1300).  Brick body
// loads depend on none of the design-variable categories of the device complex step; for shells
// the body force is linear in the section thickness (dF/dd = (dt/dd) b integral of N), and the
// gravitational and centrifugal loads, the mass residual, are differentiated by the complex step
// of the pipeline's mass term alone.
extern "C" int astro_body_load_drdd(astro_ctx *ctx, int32_t dvar, double h, int32_t kind, const double *vals,
                                    const int32_t *elements, int32_t count, const astro_state *state, double *drudd) {
    if (!ctx || !vals || !drudd || kind < 0 || kind > 2 || count < 0) return ASTRO_ERR_ARG;
    if (dvar < 1 || dvar > ctx->numDvars)
        return set_err(ctx, ASTRO_ERR_ARG, "design variable " + std::to_string(dvar) + " out of range");
    if (!(h > 0.0)) return set_err(ctx, ASTRO_ERR_ARG, "complex step h must be positive");
    const AstroPrep &P = ctx->P;
    const int n = P.n;
    if (ctx->hasShell && ctx->hasSolid) return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "body loads on mixed meshes");
    if (elements)
        for (int k = 0; k < count; ++k)
            if (elements[k] < 1 || elements[k] > P.E) return set_err(ctx, ASTRO_ERR_ARG, "element number out of range");
    if (ctx->hasSolid || (elements && count == 0)) return ASTRO_OK;
    // listed elements that depend on dvar, with multiplicity; per element dt/dd
    std::vector<int> on((size_t)P.E, 0);
    std::vector<double> dt((size_t)P.E, 0.0);
    for (int e = 0; e < P.E; ++e)
        for (int q = ctx->e2dRange[e]; q < ctx->e2dRange[e + 1]; ++q)
            if (ctx->e2d[q] == dvar) {
                on[e] = 1;
                if (ctx->dCat[dvar - 1] == ASTRO_DCAT_LAYUP_THICKNESS) dt[e] += ctx->e2c[q];
            }
    if (elements) {
        std::vector<int> cnt((size_t)P.E, 0);
        for (int k = 0; k < count; ++k) ++cnt[elements[k] - 1];
        for (int e = 0; e < P.E; ++e) on[e] *= cnt[e];
    }
    const int maxMult = *std::max_element(on.begin(), on.end());
    if (!maxMult) return ASTRO_OK;
    struct Tmp {
        DevBuf ref, li, u, iu, pa, acc, list, mult, dt;
        ~Tmp() {
            DevBuf *v[] = {&ref, &li, &u, &iu, &pa, &acc, &list, &mult, &dt};
            for (DevBuf *p : v) dev_free(*p);
        }
    } T;
    int rc;
    if ((rc = dev_alloc(ctx, T.ref, sizeof(double) * n)) || (rc = dev_alloc(ctx, T.li, sizeof(double) * n)) ||
        (rc = dev_alloc(ctx, T.acc, sizeof(double) * n)))
        return rc;
    CK(cudaMemcpyAsync(T.ref.p, drudd, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = ref_to_int_vec(ctx, dptr<double>(T.ref), dptr<double>(T.li), n))) return rc;
    CK(cudaMemsetAsync(T.acc.p, 0, sizeof(double) * n, ctx->stream));
    BodyVals bv;
    for (int k = 0; k < 7; ++k) bv.v[k] = (kind == 2 || k < 6) ? vals[k] : 0.0;
    if (kind == 0) {
        // dF/dd into acc, then li -= acc
        std::vector<int> list, ptr(1, 0);
        std::vector<double> mult;
        for (int col = 0; col < P.ncolors; ++col) {
            for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k)
                if (on[P.colorEls[k]]) {
                    list.push_back(P.colorEls[k]);
                    mult.push_back((double)on[P.colorEls[k]]);
                }
            ptr.push_back((int)list.size());
        }
        if ((rc = upload(ctx, T.list, list.data(), sizeof(int) * list.size())) ||
            (rc = upload(ctx, T.mult, mult.data(), sizeof(double) * mult.size())) ||
            (rc = upload(ctx, T.dt, dt.data(), sizeof(double) * dt.size())))
            return rc;
        for (int col = 0; col < P.ncolors; ++col) {
            const int cnt = ptr[col + 1] - ptr[col];
            if (!cnt) continue;
            k_shell_body<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(
                bv, dptr<int>(T.list) + ptr[col], cnt, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist),
                dptr<int>(ctx->d_rank), dptr<ShellProps>(ctx->d_secABD), dptr<int>(ctx->d_esec),
                dptr<int>(ctx->d_shLayRange), dptr<LayerDev>(ctx->d_shLay), nullptr, nullptr, nullptr, nullptr, nullptr,
                nullptr, dptr<double>(T.mult) + ptr[col], dptr<double>(T.dt), dptr<double>(T.acc));
        }
        k_sub<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, dptr<double>(T.acc), dptr<double>(T.li));
        if ((rc = cuda_check(ctx, cudaGetLastError(), "body load derivative"))) return rc;
    } else {
        if (state && state->node_disp) {
            DevBuf hb;
            rc = upload(ctx, hb, state->node_disp, sizeof(double) * n);
            if (!rc) rc = dev_alloc(ctx, T.u, sizeof(double) * n);
            if (!rc) rc = ref_to_int_vec(ctx, dptr<double>(hb), dptr<double>(T.u), n);
            if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "state upload");
            dev_free(hb);
            if (rc) return rc;
        } else {
            if ((rc = dev_alloc(ctx, T.u, sizeof(double) * n))) return rc;
            CK(cudaMemsetAsync(T.u.p, 0, sizeof(double) * n, ctx->stream));
        }
        const int ni = P.intVecSize;
        if (ni > 0) {
            if (state && state->internal_disp) {
                if ((rc = upload(ctx, T.iu, state->internal_disp, sizeof(double) * ni))) return rc;
            } else {
                if ((rc = dev_alloc(ctx, T.iu, sizeof(double) * ni))) return rc;
                CK(cudaMemsetAsync(T.iu.p, 0, sizeof(double) * ni, ctx->stream));
            }
        }
        std::vector<double> pa((size_t)n, 0.0);
        if (kind == 1)
            for (int r = 0; r < P.N; ++r)
                for (int c = 0; c < P.dpn; ++c) pa[(size_t)r * P.dpn + c] = -vals[c];
        if ((rc = upload(ctx, T.pa, pa.data(), sizeof(double) * n))) return rc;
        ElemDevState s1;
        s1.disp = dptr<double>(T.u);
        s1.idisp = ni > 0 ? dptr<double>(T.iu) : nullptr;
        s1.pdisp = s1.disp;
        s1.pacc = dptr<double>(T.pa);
        s1.pidisp = s1.idisp;
        s1.dynamic = 1;
        s1.beta = 0.25;
        s1.gamma = 0.5;
        s1.delT = 1.0;
        s1.massOnly = 1;
        const bool zeroState = !(state && state->node_disp);
        for (int pass = 0; pass < maxMult; ++pass) {
            std::vector<int> list, ptr(1, 0);
            for (int col = 0; col < P.ncolors; ++col) {
                for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k)
                    if (on[P.colorEls[k]] > pass) list.push_back(P.colorEls[k]);
                ptr.push_back((int)list.size());
            }
            std::function<int(const int *, int)> hook;
            if (kind == 2)
                hook = [&](const int *d_els, int cnt) {
                    k_shell_cent_pacc<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(
                        bv, d_els, cnt, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist), dptr<int>(ctx->d_rank),
                        zeroState ? nullptr : dptr<double>(T.u), dptr<double>(T.pa));
                    return cuda_check(ctx, cudaGetLastError(), "centrifugal acceleration");
                };
            if ((rc = shell4_drdd_list(ctx, dvar, h, s1, list, ptr, dptr<double>(T.acc), nullptr, hook))) return rc;
        }
        // acc = -Im(Rum(d + i h)): dF/dd = -acc / h, drudd -= dF/dd
        k_add_scaled<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, 1.0 / h, dptr<double>(T.acc), dptr<double>(T.li));
        if ((rc = cuda_check(ctx, cudaGetLastError(), "body load derivative"))) return rc;
    }
    if ((rc = int_to_ref_vec(ctx, dptr<double>(T.li), dptr<double>(T.ref), n))) return rc;
    CK(cudaMemcpyAsync(drudd, T.ref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

// ---- nodal design loads --------------------------------------------------------------------
// r_getNodeDLoad (Working/AStrO_r_designPropertyFunctions.f90:970-994, Q6 resolved: the loop runs
// over the node's own ndToD terms): the elastic nodal load of the nodeLoad design variables active
// at time t (dActTime(1) < t < dActTime(2)), one thread per node, in the internal layout (rank
// major, dpn per node).  mode 0: load += coef * d of every variable (getElasticAppliedLoad,
// Working/AStrO_commandFunctions.f90:494-502); mode 1: load -= coef for variable dvar only
// (getdRelasticdD's nodal-load branch, :1364-1373: minus the derivative of the load).
namespace {
__global__ void k_node_dload(int N, int dpn, const int *__restrict__ rank, const int *__restrict__ n2dR,
                             const int *__restrict__ n2d, const double *__restrict__ n2c, const int *__restrict__ dcat,
                             const int *__restrict__ dcomp, const double *__restrict__ dval, const double *__restrict__ act,
                             double t, int mode, int dvar, double *__restrict__ loadInt) {
    const int nd = blockIdx.x * blockDim.x + threadIdx.x;
    if (nd >= N) return;
    for (int q = n2dR[nd]; q < n2dR[nd + 1]; ++q) {
        const int d = n2d[q];
        if (dcat[d - 1] != ASTRO_DCAT_NODE_LOAD || (mode == 1 && d != dvar)) continue;
        if (act && !(t > act[2 * (d - 1)] && act[2 * (d - 1) + 1] > t)) continue;
        const int c = dcomp[d - 1];
        if (c < 1 || c > dpn) continue;  // a solid node has no rotational DOF
        const double v = mode == 0 ? n2c[q] * dval[d - 1] : -n2c[q];
        loadInt[(size_t)dpn * (rank[nd] - 1) + c - 1] += v;
    }
}
}  // namespace

static int node_dload(astro_ctx *ctx, double t, int mode, int dvar, double *vec) {
    const AstroPrep &P = ctx->P;
    const int n = P.n;
    if (ctx->n2dRange.empty()) return ASTRO_OK;
    DevBuf ref, in, act;
    int rc;
    struct Free {
        DevBuf *b[3];
        ~Free() {
            for (auto *x : b) dev_free(*x);
        }
    } fr{{&ref, &in, &act}};
    if ((rc = upload(ctx, ref, vec, sizeof(double) * n)) || (rc = dev_alloc(ctx, in, sizeof(double) * n))) return rc;
    if (!ctx->dActTime.empty() && (rc = upload(ctx, act, ctx->dActTime.data(), sizeof(double) * ctx->dActTime.size())))
        return rc;
    if ((rc = ref_to_int_vec(ctx, dptr<double>(ref), dptr<double>(in), n))) return rc;
    k_node_dload<<<(P.N + 127) / 128, 128, 0, ctx->stream>>>(
        P.N, P.dpn, dptr<int>(ctx->d_rank), dptr<int>(ctx->d_n2dR), dptr<int>(ctx->d_n2d), dptr<double>(ctx->d_n2c),
        dptr<int>(ctx->d_dCat), dptr<int>(ctx->d_dComp), dptr<double>(ctx->d_dVal),
        act.p ? dptr<double>(act) : nullptr, t, mode, dvar, dptr<double>(in));
    if ((rc = cuda_check(ctx, cudaGetLastError(), "nodal design load"))) return rc;
    if ((rc = int_to_ref_vec(ctx, dptr<double>(in), dptr<double>(ref), n))) return rc;
    CK(cudaMemcpyAsync(vec, ref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

extern "C" int astro_design_node_load(astro_ctx *ctx, double time, double *elastic_load) {
    if (!ctx || !elastic_load) return ASTRO_ERR_ARG;
    return node_dload(ctx, time, 0, 0, elastic_load);
}

extern "C" int astro_node_load_drdd(astro_ctx *ctx, int32_t dvar, double time, double *drudd) {
    if (!ctx || !drudd) return ASTRO_ERR_ARG;
    if (dvar < 1 || dvar > ctx->numDvars)
        return set_err(ctx, ASTRO_ERR_ARG, "design variable " + std::to_string(dvar) + " out of range");
    return node_dload(ctx, time, 1, dvar, drudd);
}
