// Transient design gradient: the dynamic branch of getTotaldLdD (Working/AStrO_commandFunctions.f90:
// 1411-1465) with augmentdLdu (:819-915) and the elastic branch of solveDynamicAdjoint (:917-966),
// driven over the stored states of a Newmark run.  Every element evaluation, constraint scaling,
// condensation, adjoint solve and complex step runs on the device through the library's own entry
// points; this file only orders them, as the reference's driver does.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "astro_internal.h"

namespace {

// x -> (x * 1e-20) * 1e20, the reference's scaling round trip around augmentdLdu (multFact)
void round_trip(std::vector<double> &v) {
    const double f = 1e-20;
    const double g = 1.0 / f;
    for (double &x : v) x = (x * f) * g;
}

}  // namespace

extern "C" int astro_total_dldd_transient(astro_ctx *ctx, const astro_transient_adjoint *a, double *dldd,
                                          double *disp_adj, astro_solve_stats *stats) {
    if (!ctx || !a || !dldd || !a->disp || !a->vel || !a->acc || a->num_steps < 1 || !(a->del_t > 0.0) ||
        !(a->nm_beta > 0.0) || !(a->h > 0.0))
        return ASTRO_ERR_ARG;
    astro_dims dims;
    int rc;
    if ((rc = astro_get_dims(ctx, &dims))) return rc;
    const int n = dims.el_mat_dim, ni = dims.int_vec_size, nd = ctx->numDvars, N = a->num_steps;
    const double dt = a->del_t, beta = a->nm_beta, gamma = a->nm_gamma;
    auto row = [](const double *base, int i, int len) -> std::vector<double> {
        std::vector<double> v((size_t)std::max(len, 1), 0.0);
        if (base && len > 0) std::copy(base + (size_t)i * len, base + (size_t)(i + 1) * len, v.begin());
        return v;
    };
    auto scaled = [](std::vector<double> v) {
        for (double &x : v) x *= 1e-20;
        return v;
    };
    std::vector<double> dLdu(n), dLdv(n), dLda(n), idLdu(std::max(ni, 1)), lam(n, 0.0), ilam(std::max(ni, 1), 0.0);
    std::vector<double> velAdj(n, 0.0), accAdj(n, 0.0), load(n), iload(std::max(ni, 1)), dr(n), dri(std::max(ni, 1));
    std::vector<double> mm(std::max(dims.el_mpc_size, 1)), mr(std::max(dims.el_mpc_dim, 1));
    for (int d = 0; d < nd; ++d) dldd[d] = a->dldd_explicit ? a->dldd_explicit[d] : 0.0;
    astro_solve_stats acc{};
    for (int i = N; i >= 1; --i) {
        std::fill(dLdu.begin(), dLdu.end(), 0.0);
        std::fill(dLdv.begin(), dLdv.end(), 0.0);
        std::fill(dLda.begin(), dLda.end(), 0.0);
        std::fill(idLdu.begin(), idLdu.end(), 0.0);
        // the state of step i (node) after the round trip of the previous augment
        std::vector<double> u = row(a->disp, i, n), v = row(a->vel, i, n), ac = row(a->acc, i, n),
                            iu = row(a->int_disp, i, ni);
        if (i < N) {
            // augmentdLdu at node = state i+1, prev = state i, all scaled by 1e-20
            std::vector<double> nu = scaled(row(a->disp, i + 1, n)), nv = scaled(row(a->vel, i + 1, n)),
                                na = scaled(row(a->acc, i + 1, n)), niu = scaled(row(a->int_disp, i + 1, ni));
            std::vector<double> pu = scaled(u), pv = scaled(v), pa = scaled(ac), piu = scaled(iu);
            astro_state st{};
            st.node_disp = nu.data();
            st.node_vel = nv.data();
            st.node_acc = na.data();
            st.internal_disp = niu.data();
            st.prev_vel = pv.data();
            st.prev_acc = pa.data();
            st.dynamic = 1;
            st.nm_beta = beta;
            st.nm_gamma = gamma;
            st.del_t = dt;
            // block 3: prevDisp = dispAdj, prevIntDisp = intDispAdj
            st.prev_disp = lam.data();
            st.prev_int_disp = ilam.data();
            std::fill(load.begin(), load.end(), 0.0);
            std::fill(iload.begin(), iload.end(), 0.0);
            if ((rc = astro_el_soln_load(ctx, 0, &st, load.data(), iload.data(), nullptr, nullptr, nullptr))) return rc;
            for (int k = 0; k < n; ++k) dLdu[k] += load[k] + accAdj[k];
            for (int k = 0; k < ni; ++k) idLdu[k] += iload[k];
            // block 4: prevAcc = dispAdj
            st.prev_disp = pu.data();
            st.prev_int_disp = piu.data();
            st.prev_acc = lam.data();
            std::fill(load.begin(), load.end(), 0.0);
            std::fill(iload.begin(), iload.end(), 0.0);
            if ((rc = astro_el_soln_load(ctx, 0, &st, load.data(), iload.data(), nullptr, nullptr, nullptr))) return rc;
            for (int k = 0; k < n; ++k)
                dLda[k] += load[k] + 0.5 * dt * dt * (1.0 - 2.0 * beta) * accAdj[k] + dt * (1.0 - gamma) * velAdj[k];
            // block 5: prevVel = dispAdj
            st.prev_acc = pa.data();
            st.prev_vel = lam.data();
            std::fill(load.begin(), load.end(), 0.0);
            std::fill(iload.begin(), iload.end(), 0.0);
            if ((rc = astro_el_soln_load(ctx, 0, &st, load.data(), iload.data(), nullptr, nullptr, nullptr))) return rc;
            for (int k = 0; k < n; ++k) dLdv[k] += load[k] + dt * accAdj[k] + velAdj[k];
            round_trip(u);
            round_trip(v);
            round_trip(ac);
            round_trip(iu);
        }
        // getdObjdU at t_i
        for (int k = 0; k < n; ++k) {
            if (a->dldu) dLdu[k] += a->dldu[(size_t)(i - 1) * n + k];
            if (a->dldv) dLdv[k] += a->dldv[(size_t)(i - 1) * n + k];
            if (a->dlda) dLda[k] += a->dlda[(size_t)(i - 1) * n + k];
        }
        if (a->int_dldu)
            for (int k = 0; k < ni; ++k) idLdu[k] += a->int_dldu[(size_t)(i - 1) * ni + k];
        // solveDynamicAdjoint at node = state i, prev = state i-1
        for (int k = 0; k < n; ++k) {
            velAdj[k] = dLdv[k];
            accAdj[k] = (-1.0 / (dt * dt * beta)) * (dLda[k] + dt * gamma * velAdj[k]);
            dLdu[k] -= accAdj[k];
        }
        std::vector<double> pu = row(a->disp, i - 1, n), pv = row(a->vel, i - 1, n), pa = row(a->acc, i - 1, n),
                            piu = row(a->int_disp, i - 1, ni);
        astro_state st{};
        st.node_disp = u.data();
        st.node_vel = v.data();
        st.node_acc = ac.data();
        st.internal_disp = iu.data();
        st.prev_disp = pu.data();
        st.prev_vel = pv.data();
        st.prev_acc = pa.data();
        st.prev_int_disp = piu.data();
        st.dynamic = 1;
        st.nm_beta = beta;
        st.nm_gamma = gamma;
        st.del_t = dt;
        std::fill(load.begin(), load.end(), 0.0);
        std::fill(iload.begin(), iload.end(), 0.0);
        if ((rc = astro_el_soln_load(ctx, 1, &st, load.data(), iload.data(), nullptr, nullptr, nullptr))) return rc;
        if ((rc = astro_scale_mpc(ctx, mm.data(), mr.data()))) return rc;
        if (ni > 0 && (rc = astro_update_external_rhs(ctx, dLdu.data(), idLdu.data()))) return rc;
        astro_solve_stats s{};
        rc = astro_solve_static(ctx, dLdu.data(), lam.data(), &a->solve, &s);  // warm start from the last adjoint
        acc.iterations += s.iterations;
        acc.restarts += s.restarts;
        acc.refinements += s.refinements;
        acc.seconds += s.seconds;
        acc.rel_residual = std::max(acc.rel_residual, s.rel_residual);
        acc.conditional_graph = s.conditional_graph;
        acc.residual_kind = s.residual_kind;
        if (rc) {
            acc.status = rc;
            if (stats) *stats = acc;
            return rc;
        }
        if (ni > 0 && (rc = astro_update_internal_soln(ctx, lam.data(), ilam.data(), idLdu.data()))) return rc;
        for (int d = 1; d <= nd; ++d) {
            if ((rc = astro_drdd_complex(ctx, d, a->h, &st, dr.data(), dri.data()))) return rc;
            double s1 = 0.0, s2 = 0.0;
            for (int k = 0; k < n; ++k) s1 += lam[k] * dr[k];
            for (int k = 0; k < ni; ++k) s2 += ilam[k] * dri[k];
            dldd[d - 1] -= s1 + s2;
        }
    }
    if (disp_adj) std::copy(lam.begin(), lam.end(), disp_adj);
    acc.status = ASTRO_OK;
    if (stats) *stats = acc;
    return ASTRO_OK;
}

// ---- solution-history step files ---------------------------------------------------------------

namespace {

// one Fortran unformatted sequential record: 4-byte length, data, 4-byte length
bool put_record(FILE *f, const double *v, int count) {
    const uint32_t len = (uint32_t)(sizeof(double) * (size_t)count);
    std::vector<double> z;
    if (!v) {
        z.assign((size_t)count, 0.0);
        v = z.data();
    }
    return fwrite(&len, 4, 1, f) == 1 && (count == 0 || fwrite(v, sizeof(double), (size_t)count, f) == (size_t)count) &&
           fwrite(&len, 4, 1, f) == 1;
}

// reads the next record into v (its first count values; a longer record is read in part, as a
// Fortran list read of a shorter array does); false when it is missing or shorter
bool get_record(FILE *f, double *v, int count) {
    uint32_t len = 0, tail = 0;
    if (fread(&len, 4, 1, f) != 1) return false;
    const size_t want = sizeof(double) * (size_t)count;
    if (len < want) return false;
    std::vector<double> buf(len / sizeof(double) + 1);
    if (len > 0 && fread(buf.data(), 1, len, f) != len) return false;
    if (fread(&tail, 4, 1, f) != 1 || tail != len) return false;
    if (v && count > 0) std::copy(buf.begin(), buf.begin() + count, v);
    return true;
}

}  // namespace

extern "C" int astro_write_step_file(const char *path, int32_t num_nodes, int32_t el_mat_dim, int32_t int_vec_size,
                                     const double *prev_temp, const double *prev_tdot, const double *prev_disp,
                                     const double *prev_int_disp, const double *prev_vel, const double *prev_acc) {
    if (!path || num_nodes < 0 || el_mat_dim < 0 || int_vec_size < 0 || !prev_disp || !prev_vel || !prev_acc)
        return ASTRO_ERR_ARG;
    FILE *f = fopen(path, "wb");
    if (!f) return ASTRO_ERR_ARG;
    bool ok = put_record(f, prev_temp, num_nodes) && put_record(f, prev_tdot, num_nodes) &&
              put_record(f, prev_disp, el_mat_dim);
    if (ok && int_vec_size >= 1) ok = put_record(f, prev_int_disp, int_vec_size);
    ok = ok && put_record(f, prev_vel, el_mat_dim) && put_record(f, prev_acc, el_mat_dim);
    ok = (fclose(f) == 0) && ok;
    return ok ? ASTRO_OK : ASTRO_ERR_ARG;
}

extern "C" int astro_read_step_file(const char *path, int32_t num_nodes, int32_t el_mat_dim, int32_t int_vec_size,
                                    double *prev_temp, double *prev_tdot, double *prev_disp, double *prev_int_disp,
                                    double *prev_vel, double *prev_acc) {
    if (!path || num_nodes < 0 || el_mat_dim < 0 || int_vec_size < 0) return ASTRO_ERR_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) return ASTRO_ERR_ARG;
    bool ok = get_record(f, prev_temp, num_nodes) && get_record(f, prev_tdot, num_nodes) &&
              get_record(f, prev_disp, el_mat_dim);
    if (ok && int_vec_size > 1) ok = get_record(f, prev_int_disp, int_vec_size);
    ok = ok && get_record(f, prev_vel, el_mat_dim) && get_record(f, prev_acc, el_mat_dim);
    fclose(f);
    return ok ? ASTRO_OK : ASTRO_ERR_ARG;
}
