// The reference's output files (vm.out, err.out, *.iout) from an RVE handle
// (voce_io.h).  Host code over the public ABI: fields come down through
// voce_rve_get_field; the byte layouts are those of io.c's MPI-IO writers.
#include "voce_io.h"
#include "voce_internal.h"

#include <fcntl.h>
#include <unistd.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

int fail_io(int code, const std::string &msg) { return voce::set_error(code, msg.c_str()); }

// Open like MPI_File_open(MPI_MODE_CREATE|MPI_MODE_WRONLY): create if absent,
// no truncation, write from offset 0.
int write_file(const std::string &path, const void *data, size_t n)
{
    const int fd = ::open(path.c_str(), O_WRONLY | O_CREAT, 0666);
    if (fd < 0) return fail_io(VOCE_ERR_IO, "cannot open " + path);
    const char *p = static_cast<const char *>(data);
    size_t done = 0;
    while (done < n) {
        const ssize_t w = ::write(fd, p + done, n - done);
        if (w <= 0) {
            ::close(fd);
            return fail_io(VOCE_ERR_IO, "cannot write " + path);
        }
        done += (size_t)w;
    }
    if (::close(fd) != 0) return fail_io(VOCE_ERR_IO, "cannot close " + path);
    return VOCE_OK;
}

std::string fmt_name(const char *pattern, const char *name, int a, int b = -1)
{
    char buf[1024];
    if (b < 0) std::snprintf(buf, sizeof(buf), pattern, name, a);
    else std::snprintf(buf, sizeof(buf), pattern, name, a, b);
    return buf;
}

struct Dims {
    int nx, ny, nz;
    long long nv;
};

int rve_dims(voce_rve *r, Dims *d)
{
    voce_namelist nl;
    const int rc = voce_rve_get_namelist(r, &nl);
    if (rc) return rc;
    d->nx = nl.CellDim[0];
    d->ny = nl.CellDim[1];
    d->nz = nl.CellDim[2];
    d->nv = (long long)d->nx * d->ny * d->nz;
    return VOCE_OK;
}

int get(voce_rve *r, int field, long long n, std::vector<double> &out)
{
    out.resize((size_t)n);
    return voce_rve_get_field(r, field, out.data());
}

// Component i of the Voigt order 11,22,33,23,13,12 of a row-major 3x3.
inline int voigt_row(int i) { static const int a[6] = {0, 1, 2, 1, 0, 0}; return a[i]; }
inline int voigt_col(int i) { static const int b[6] = {0, 1, 2, 2, 2, 1}; return b[i]; }

// Sym(DisGrad) - Eps in that order (io.c:289-302).
inline double els_comp(const double *D, const double *E, int i)
{
    const int a = voigt_row(i), b = voigt_col(i);
    if (i < 3) return D[3 * a + a] - E[3 * a + a];
    return (D[3 * a + b] + D[3 * b + a]) / 2.0 - E[3 * a + b];
}

// The Lebensohn-Tome basis of chg_basis (kinematics.c:33-56), B[p][i][j].
void lt_basis(double B[6][3][3])
{
    const double r2 = 0.70710678118654744, r3 = 0.57735026918962584, r6 = 0.40824829046386304;
    std::memset(B, 0, sizeof(double) * 54);
    B[0][0][0] = -r2; B[0][1][1] = r2;
    B[1][0][0] = -r6; B[1][1][1] = -r6; B[1][2][2] = 2. * r6;
    B[2][1][2] = r2; B[2][2][1] = r2;
    B[3][0][2] = r2; B[3][2][0] = r2;
    B[4][0][1] = r2; B[4][1][0] = r2;
    B[5][0][0] = r3; B[5][1][1] = r3; B[5][2][2] = r3;
}

// Bunge angles in degrees of a sample->crystal matrix: the matrix->angles
// branch of EulerToTransMatrix (kinematics.c:197-215), with the reference's
// value of pi (evp.h:52).
void bunge_from_matrix(const double a[3][3], double *t1, double *ph, double *t2)
{
    const double pi_ref = 3.14159265359;
    double p = std::acos(a[2][2]), u, w;
    if (std::fabs(a[2][2]) > 0.9999) {
        w = 0.;
        u = std::atan2(a[0][1], a[0][0]);
    } else {
        const double sph = std::sin(p);
        u = std::atan2(a[2][0] / sph, -1.0 * a[2][1] / sph);
        w = std::atan2(a[0][2] / sph, a[1][2] / sph);
    }
    p *= 180. / pi_ref;
    u *= 180. / pi_ref;
    w *= 180. / pi_ref;
    *t1 = u;
    *ph = p;
    *t2 = w;
}

// Six component files of a 3x3 field (eps, sig, edot, els).
int write_six(voce_rve *r, const Dims &dm, int kind, const char *name, int step)
{
    const long long nv = dm.nv;
    std::vector<double> buf((size_t)nv);
    int rc;
    if (kind == VOCE_IOUT_SIG || kind == VOCE_IOUT_EDOT) {
        std::vector<double> f;
        if ((rc = get(r, kind == VOCE_IOUT_SIG ? VOCE_FIELD_SIG_VOIGT : VOCE_FIELD_EDOT_VOIGT, 6 * nv, f)))
            return rc;
        for (int i = 0; i < 6; ++i) {
            const std::string fn = fmt_name("%s_%01d_S%04d.iout", name, i + 1, step);
            if ((rc = write_file(fn, f.data() + (size_t)i * nv, sizeof(double) * nv))) return rc;
        }
        return VOCE_OK;
    }
    std::vector<double> E;
    if ((rc = get(r, VOCE_FIELD_EPS, 9 * nv, E))) return rc;
    std::vector<double> D;
    if (kind == VOCE_IOUT_ELS && (rc = get(r, VOCE_FIELD_DISGRAD, 9 * nv, D))) return rc;
    for (int i = 0; i < 6; ++i) {
        const int a = voigt_row(i), b = voigt_col(i);
        for (long long v = 0; v < nv; ++v)
            buf[v] = kind == VOCE_IOUT_ELS ? els_comp(&D[9 * v], &E[9 * v], i) : E[9 * v + 3 * a + b];
        const char *pat = kind == VOCE_IOUT_ELS ? "%s_%01d_S%06d.iout" : "%s_%01d_S%04d.iout";
        if ((rc = write_file(fmt_name(pat, name, i + 1, step), buf.data(), sizeof(double) * nv))) return rc;
    }
    return VOCE_OK;
}

// {int grain; 12 doubles} records (io.c:651-937): the MPI struct type puts the
// doubles at offset 8, so bytes 4..7 are a hole; 104 bytes a record.
int write_sys_records(voce_rve *r, const Dims &dm, int field, const char *name, int step)
{
    const long long nv = dm.nv;
    std::vector<double> f;
    int rc;
    if ((rc = get(r, field, 12 * nv, f))) return rc;
    std::vector<int> grain((size_t)nv);
    if ((rc = voce_rve_get_ids(r, grain.data(), nullptr))) return rc;
    const size_t rec = 104;
    std::vector<unsigned char> out((size_t)nv * rec, 0);
    for (long long v = 0; v < nv; ++v) {
        unsigned char *p = out.data() + (size_t)v * rec;
        const int32_t g = grain[v];
        std::memcpy(p, &g, 4);
        std::memcpy(p + 8, &f[12 * v], 12 * sizeof(double));
    }
    return write_file(fmt_name("%s_S%04d.iout", name, step), out.data(), out.size());
}

// {double angle[3]; int coord[3], jgr, jph, buff} records (io.c:939-1003), 48 bytes.
int write_texture(voce_rve *r, const Dims &dm, const char *name, int step)
{
    const long long nv = dm.nv;
    std::vector<double> T;
    int rc;
    if ((rc = get(r, VOCE_FIELD_TRANMAT, 9 * nv, T))) return rc;
    std::vector<int> grain((size_t)nv), phase((size_t)nv);
    if ((rc = voce_rve_get_ids(r, grain.data(), phase.data()))) return rc;
    const size_t rec = 48;
    std::vector<unsigned char> out((size_t)nv * rec, 0);
    long long v = 0;
    for (int x = 0; x < dm.nx; ++x)
        for (int y = 0; y < dm.ny; ++y)
            for (int z = 0; z < dm.nz; ++z, ++v) {
                double sa2xt[3][3], ang[3];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) sa2xt[a][b] = T[9 * v + 3 * b + a];
                bunge_from_matrix(sa2xt, &ang[0], &ang[1], &ang[2]);
                const int32_t ints[6] = {x + 1, y + 1, z + 1, grain[v], phase[v], 0};
                unsigned char *p = out.data() + (size_t)v * rec;
                std::memcpy(p, ang, 24);
                std::memcpy(p + 24, ints, 24);
            }
    return write_file(fmt_name("%s_S%04d.iout", name, step), out.data(), out.size());
}

// 0.5 Sig : T(els) with T the basis expansion of the Voigt-ordered elastic
// strain (io.c:246-262).
int write_work_e(voce_rve *r, const Dims &dm, const char *name, int step)
{
    const long long nv = dm.nv;
    std::vector<double> S, D, E;
    int rc;
    if ((rc = get(r, VOCE_FIELD_SIG, 9 * nv, S))) return rc;
    if ((rc = get(r, VOCE_FIELD_DISGRAD, 9 * nv, D))) return rc;
    if ((rc = get(r, VOCE_FIELD_EPS, 9 * nv, E))) return rc;
    double B[6][3][3];
    lt_basis(B);
    std::vector<double> out((size_t)nv);
    for (long long v = 0; v < nv; ++v) {
        double els[6], acc = 0.0;
        for (int i = 0; i < 6; ++i) els[i] = els_comp(&D[9 * v], &E[9 * v], i);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double t = 0.0;
                for (int i = 0; i < 6; ++i) t += els[i] * B[i][a][b];
                acc += 0.5 * S[9 * v + 3 * a + b] * t;
            }
        out[v] = acc;
    }
    return write_file(fmt_name("%s_S%06d.iout", name, step), out.data(), sizeof(double) * nv);
}

int write_scalar(voce_rve *r, const Dims &dm, int field, const char *pattern, const char *name, int step)
{
    std::vector<double> f;
    int rc;
    if ((rc = get(r, field, dm.nv, f))) return rc;
    return write_file(fmt_name(pattern, name, step), f.data(), sizeof(double) * dm.nv);
}

std::string join(const char *dir, const char *name)
{
    if (!dir || !dir[0]) return name;
    std::string s(dir);
    if (s.back() != '/') s += '/';
    return s + name;
}

}  // namespace

extern "C" {

int voce_rve_write_iout(voce_rve *r, int kind, const char *name, int step)
{
    if (!r || !name) return fail_io(VOCE_ERR_ARG, "null argument");
    Dims dm;
    int rc = rve_dims(r, &dm);
    if (rc) return rc;
    switch (kind) {
    case VOCE_IOUT_EPS: case VOCE_IOUT_SIG: case VOCE_IOUT_ELS: case VOCE_IOUT_EDOT:
        return write_six(r, dm, kind, name, step);
    case VOCE_IOUT_SLIP: return write_sys_records(r, dm, VOCE_FIELD_GAMMATOTAL, name, step);
    case VOCE_IOUT_TAUX: return write_sys_records(r, dm, VOCE_FIELD_TAUX, name, step);
    case VOCE_IOUT_CRSS: return write_sys_records(r, dm, VOCE_FIELD_CRSS, name, step);
    case VOCE_IOUT_TEX: return write_texture(r, dm, name, step);
    case VOCE_IOUT_SVM: return write_scalar(r, dm, VOCE_FIELD_SVM, "%s_S%04d.iout", name, step);
    case VOCE_IOUT_EVM: return write_scalar(r, dm, VOCE_FIELD_EVM, "%s_S%04d.iout", name, step);
    case VOCE_IOUT_RHO_RSS: return write_scalar(r, dm, VOCE_FIELD_RHO_RSS, "%s_S%04d.iout", name, step);
    case VOCE_IOUT_RHO_CRSS: return write_scalar(r, dm, VOCE_FIELD_RHO_CRSS, "%s_S%04d.iout", name, step);
    case VOCE_IOUT_WORK_P: return write_scalar(r, dm, VOCE_FIELD_WORK_P, "%s_S%06d.iout", name, step);
    case VOCE_IOUT_WORK_E: return write_work_e(r, dm, name, step);
    case VOCE_IOUT_NEW_POSITION: {
        // 24-byte records of three doubles (io.c:806-858), here the corrected
        // displacement fluctuation (VOCE_FIELD_DISP_FLUCT)
        std::vector<double> f;
        if ((rc = get(r, VOCE_FIELD_DISP_FLUCT, 3 * dm.nv, f))) return rc;
        return write_file(fmt_name("%s_S%04d.iout", name, step), f.data(), sizeof(double) * 3 * dm.nv);
    }
    default: return fail_io(VOCE_ERR_ARG, "unknown .iout kind " + std::to_string(kind));
    }
}

int voce_rve_write_step_iout(voce_rve *r, int istep, const char *dir)
{
    voce_namelist nl;
    int rc = voce_rve_get_namelist(r, &nl);
    if (rc) return rc;
    // evolution.c:569: PrintControl[1] <= 0 selects no increment here (the
    // reference would divide by zero)
    if (nl.PrintControl[0] != 1 || nl.PrintControl[1] <= 0 ||
        istep / nl.PrintControl[1] * nl.PrintControl[1] != istep)
        return VOCE_OK;
    static const struct { int kind; const char *name; } base[] = {
        {VOCE_IOUT_EPS, "eps"}, {VOCE_IOUT_SIG, "sig"}, {VOCE_IOUT_ELS, "els"}, {VOCE_IOUT_EDOT, "edot"}};
    static const struct { int kind; const char *name; } tex[] = {
        {VOCE_IOUT_SLIP, "slip_sys"}, {VOCE_IOUT_TAUX, "taux_sys"}, {VOCE_IOUT_CRSS, "crss_sys"},
        {VOCE_IOUT_TEX, "tex"}, {VOCE_IOUT_RHO_RSS, "rho_rss"}, {VOCE_IOUT_RHO_CRSS, "rho_crss"},
        {VOCE_IOUT_WORK_P, "work_p"}, {VOCE_IOUT_SVM, "SVM"}, {VOCE_IOUT_EVM, "EVM"},
        {VOCE_IOUT_NEW_POSITION, "new_position"}};
    for (const auto &w : base)
        if ((rc = voce_rve_write_iout(r, w.kind, join(dir, w.name).c_str(), istep))) return rc;
    if (nl.Tex_Flag == 1)
        for (const auto &w : tex)
            if ((rc = voce_rve_write_iout(r, w.kind, join(dir, w.name).c_str(), istep))) return rc;
    return VOCE_OK;
}

int voce_rve_write_final_iout(voce_rve *r, const char *dir)
{
    voce_namelist nl;
    int rc = voce_rve_get_namelist(r, &nl);
    if (rc) return rc;
    if (nl.Tex_Flag != 1) return VOCE_OK;
    static const struct { int kind; const char *name; } fin[] = {
        {VOCE_IOUT_SLIP, "slip_final"}, {VOCE_IOUT_TAUX, "taux_final"}, {VOCE_IOUT_CRSS, "crss_final"},
        {VOCE_IOUT_TEX, "tex_final"}, {VOCE_IOUT_SVM, "SVM_final"}, {VOCE_IOUT_EVM, "EVM_final"},
        {VOCE_IOUT_RHO_RSS, "rho_rss_final"}, {VOCE_IOUT_RHO_CRSS, "rho_crss_final"},
        {VOCE_IOUT_WORK_P, "work_p_final"}, {VOCE_IOUT_WORK_E, "work_e_final"},
        {VOCE_IOUT_EPS, "eps_final"}, {VOCE_IOUT_SIG, "sig_final"},
        {VOCE_IOUT_NEW_POSITION, "new_position_final"}, {VOCE_IOUT_EDOT, "edot_final"},
        {VOCE_IOUT_ELS, "els_final"}};
    for (const auto &w : fin)
        if ((rc = voce_rve_write_iout(r, w.kind, join(dir, w.name).c_str(), 0))) return rc;
    return VOCE_OK;
}

int voce_write_log_headers(FILE *fp_vm, FILE *fp_err)
{
    if (fp_vm) std::fprintf(fp_vm, "EVM\tEVMP\tDVM\tDVMP\tSVM\tSVMSVM_1\tIteration_tot\n");
    if (fp_err) std::fprintf(fp_err, "IT\tERRE\tERRS\tSVM\n");
    return VOCE_OK;
}

int voce_rve_write_log(const voce_rve *r, int k, int n_steps, FILE *fp_vm, FILE *fp_err)
{
    if (!r) return fail_io(VOCE_ERR_ARG, "null argument");
    voce_increment rec;
    int rc = voce_rve_get_increment(r, k, &rec);
    if (rc) return rc;
    if (fp_err) {
        std::vector<double> ee((size_t)rec.iters + 1), es(ee.size()), sv(ee.size());
        const int n = voce_rve_get_iter_log(r, k, ee.data(), es.data(), sv.data(), (int)ee.size());
        if (n < 0) return -n;
        if (n_steps != 1) std::fprintf(fp_err, "STEP = %d\n", rec.istep);
        for (int i = 0; i < n; ++i) std::fprintf(fp_err, "%d\t%e\t%e\t%e\n", i + 1, ee[i], es[i], sv[i]);
        std::fflush(fp_err);
    }
    if (fp_vm) {
        std::fprintf(fp_vm, "%e\t%e\t%e\t%e\t%e\t%e\t%d\n", rec.e_vm, rec.evmp, rec.d_vm, rec.dvmp,
                     rec.s_vm, rec.s_vm1, rec.iter_total);
        std::fflush(fp_vm);
    }
    return VOCE_OK;
}

}  // extern "C"
