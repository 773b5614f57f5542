// gi_formats.cpp -- the Giant-Impact setup, parameter, statistics and body
// files, read and written in the reference drivers' formats, and the host
// steps of building bodies and setting up an impact.
//
// Text setup files are parsed as the reference parses them: for each value
// in a fixed order, skip past the next '=' and read one number with the
// type of the reference's variable (getline(data, name, '=') then
// data >> value in generateTargetImpactor.cu:169-248,
// impactInitialization.cu:183-217, impactAddTime.cu:60-102 and
// impactBasicFunctions.h:31-107).  Key names are not checked, exactly as in
// the reference.  Binary files use the reference's raw layouts:
//   targetImpactorInitialPosVel: int N, N float4 pos, N float4 vel
//     (generateTargetImpactorBasicFunctions.h:713-722)
//   impactPosVel: frames of float time, N float4 pos, N float4 vel
//     (impactInitialization.cu:373-378, impactAddTime.cu:424-428)
//
// The host arithmetic of the body builder and of the initial statistics
// keeps the reference's types (float positions, double sums in index
// order); this file is compiled with -ffp-contract=off so that it rounds as
// the reference's host code does, on x86-64 and aarch64 alike.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gi_api.h"
#include "gi_host.h"

namespace {

constexpr double kPi = 3.141592654;                // commonSetup.h:29
constexpr double kUniversalGravity = 6.67408e-20;  // km^3 kg^-1 s^-2, commonSetup.h:31
constexpr double kMassOfEarth = 5.97219e24;        // kg, commonSetup.h:33
constexpr double kRadiusOfEarth = 6378.0;          // km, commonSetup.h:35

bool slurp(const char *path, std::string &out)
{
    FILE *f = path ? std::fopen(path, "rb") : nullptr;
    if (!f) return false;
    char buf[65536];
    size_t k;
    out.clear();
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, k);
    std::fclose(f);
    return true;
}

// Sequential "skip past '=' then read one number" reader.
struct OrderedReader {
    const std::string &s;
    size_t at = 0;
    bool ok = true;
    explicit OrderedReader(const std::string &text) : s(text) {}
    const char *value_start()
    {
        if (!ok) return nullptr;
        const size_t eq = s.find('=', at);
        if (eq == std::string::npos) { ok = false; return nullptr; }
        at = eq + 1;
        while (at < s.size() && std::isspace((unsigned char)s[at])) ++at;
        return s.c_str() + at;
    }
    template <class T, class F> T parse(F conv)
    {
        const char *p = value_start();
        if (!p) return T(0);
        char *end = nullptr;
        errno = 0;
        const T v = conv(p, &end);
        if (end == p) { ok = false; return T(0); }
        at += (size_t)(end - p);
        return v;
    }
    double d() { return parse<double>([](const char *p, char **e) { return std::strtod(p, e); }); }
    float f() { return parse<float>([](const char *p, char **e) { return std::strtof(p, e); }); }
    int i()
    {
        return parse<int>([](const char *p, char **e) { return (int)std::strtol(p, e, 10); });
    }
};

int open_text(const char *path, std::string &t)
{
    if (!path) return GI_ERR_INVALID_ARG;
    return slurp(path, t) ? GI_OK : GI_ERR_IO;
}

// Cube root by Newton's method from above with +, -, *, / only, so the
// result is the same on every host (libm's pow / cbrt need not be).
double cbrt_det(double x)
{
    if (!(x > 0.0)) return 0.0;
    double y = x > 1.0 ? x : 1.0;
    for (int it = 0; it < 400; ++it) {
        const double next = y - (y * y * y - x) / (3.0 * y * y);
        if (!(next < y)) break;
        y = next;
    }
    return y;
}

// Body index ranges of the builder order [Fe1, Si1, Fe2, Si2].
struct BodyRanges {
    int fe0, fe1, si0, si1;
};
BodyRanges body_ranges(const gi_body_params &b, int body)
{
    if (body == 1) return {0, b.nfe1, b.nfe1, b.nfe1 + b.nsi1};
    const int o = b.nfe1 + b.nsi1;
    return {o, o + b.nfe2, o + b.nfe2, o + b.nfe2 + b.nsi2};
}

bool counts_ok(const gi_body_params &b)
{
    return b.n >= 0 && b.nfe1 >= 0 && b.nsi1 >= 0 && b.nfe2 >= 0 && b.nsi2 >= 0 &&
           (long long)b.nfe1 + b.nsi1 + b.nfe2 + b.nsi2 == b.n;
}

// getCenterOfMass / getAverageLinearVelocity of one body in the builder
// order (generateTargetImpactorBasicFunctions.h:29-80, :119-171): double sums
// in index order divided by the setup's body mass MassOfBody1/2.
void body_mean(const float *a, const gi_generation_plan &pl, int body, double out[3])
{
    const gi_body_params &b = pl.body;
    const double total = body == 1 ? pl.mass_body1 : pl.mass_body2;
    out[0] = out[1] = out[2] = 0.0;
    if (total < 0.00000000001) return;
    const BodyRanges r = body_ranges(b, body);
    for (int i = r.fe0; i < r.fe1; ++i)
        for (int c = 0; c < 3; ++c) out[c] += a[4 * (size_t)i + c] * b.mass_fe;
    for (int i = r.si0; i < r.si1; ++i)
        for (int c = 0; c < 3; ++c) out[c] += a[4 * (size_t)i + c] * b.mass_si;
    for (int c = 0; c < 3; ++c) out[c] /= total;
}

// getAngularMomentum (generateTargetImpactorBasicFunctions.h:173-237).
void body_angular_momentum(const float *pos, const float *vel, const gi_generation_plan &pl,
                           int body, double out[3])
{
    const gi_body_params &b = pl.body;
    double c[3], u[3];
    body_mean(pos, pl, body, c);
    body_mean(vel, pl, body, u);
    out[0] = out[1] = out[2] = 0.0;
    const BodyRanges r = body_ranges(b, body);
    auto add = [&](int i, double m) {
        const float *p = pos + 4 * (size_t)i, *v = vel + 4 * (size_t)i;
        const double rx = p[0] - c[0], ry = p[1] - c[1], rz = p[2] - c[2];
        const double vx = v[0] - u[0], vy = v[1] - u[1], vz = v[2] - u[2];
        out[0] += (ry * vz - rz * vy) * m;
        out[1] += -(rx * vz - rz * vx) * m;
        out[2] += (rx * vy - ry * vx) * m;
    };
    for (int i = r.fe0; i < r.fe1; ++i) add(i, b.mass_fe);
    for (int i = r.si0; i < r.si1; ++i) add(i, b.mass_si);
}

// getRadiusOfBody (generateTargetImpactorBasicFunctions.h:82-117); the
// reference leaves the running maximum uninitialised, here it starts at 0.
double body_radius(const float *pos, const gi_generation_plan &pl, int body)
{
    double c[3];
    body_mean(pos, pl, body, c);
    const BodyRanges r = body_ranges(pl.body, body);
    double radius = 0.0;
    for (int i = r.fe0; i < r.si1; ++i) {
        const double x = (double)pos[4 * (size_t)i] - c[0];
        const double y = (double)pos[4 * (size_t)i + 1] - c[1];
        const double z = (double)pos[4 * (size_t)i + 2] - c[2];
        const double d = std::sqrt(x * x + y * y + z * z);
        if (d > radius) radius = d;
    }
    return radius;
}

// Cell lists over one material group for the builder's redraw test.
struct GroupGrid {
    std::unordered_map<uint64_t, int> head;
    std::vector<int> next;  // by body index - base
    static int cell(float x) { return (int)std::floor(x); }
    static uint64_t key(int cx, int cy, int cz)
    {
        return ((uint64_t)(uint32_t)cx << 42) ^ ((uint64_t)(uint32_t)cy << 21) ^ (uint32_t)cz;
    }
};

}  // namespace

// ------------------------------------------------------------ setup files --

extern "C" int gi_read_setup_generating(const char *path, gi_setup_generating *o)
{
    if (!o) return GI_ERR_INVALID_ARG;
    std::string t;
    if (int st = open_text(path, t)) return st;
    OrderedReader r(t);
    for (int k = 0; k < 4; ++k) o->spin1[k] = r.f();
    for (int k = 0; k < 4; ++k) o->spin2[k] = r.f();
    o->frac_earth_mass1 = r.d();
    o->frac_earth_mass2 = r.d();
    o->frac_fe1 = r.d();
    o->frac_si1 = r.d();
    o->frac_fe2 = r.d();
    o->frac_si2 = r.d();
    o->damp1 = r.f();
    o->damp2 = r.f();
    o->n = r.i();
    o->damp_time = r.d();
    o->damp_rest_time = r.d();
    o->spin_rest_time = r.d();
    o->dt = r.d();
    o->density_fe = r.d();
    o->density_si = r.d();
    o->k_fe = r.d();
    o->k_si = r.d();
    o->kr_fe = r.d();
    o->kr_si = r.d();
    o->sd_fe = r.d();
    o->sd_si = r.d();
    o->draw_rate = r.i();
    return r.ok ? GI_OK : GI_ERR_FORMAT;
}

extern "C" int gi_read_setup_impact_init(const char *path, gi_setup_impact_init *o)
{
    if (!o) return GI_ERR_INVALID_ARG;
    std::string t;
    if (int st = open_text(path, t)) return st;
    OrderedReader r(t);
    for (int k = 0; k < 3; ++k) o->pos1[k] = r.f();
    for (int k = 0; k < 3; ++k) o->pos2[k] = r.f();
    for (int k = 0; k < 3; ++k) o->vel1[k] = r.f();
    for (int k = 0; k < 3; ++k) o->vel2[k] = r.f();
    return r.ok ? GI_OK : GI_ERR_FORMAT;
}

extern "C" int gi_read_setup_add_time(const char *path, gi_setup_add_time *o)
{
    if (!o) return GI_ERR_INVALID_ARG;
    std::string t;
    if (int st = open_text(path, t)) return st;
    OrderedReader r(t);
    o->additional_time_days = r.d();
    o->dt = r.d();
    o->draw_rate = r.i();
    o->record_rate = r.i();
    o->recenter_rate = r.i();
    return r.ok ? GI_OK : GI_ERR_FORMAT;
}

extern "C" int gi_read_body_params(const char *path, gi_body_params *o)
{
    if (!o) return GI_ERR_INVALID_ARG;
    std::string t;
    if (int st = open_text(path, t)) return st;
    OrderedReader r(t);
    o->unit_time = r.d();
    o->unit_length = r.d();
    o->unit_mass = r.d();
    o->mass_fe = r.d();
    o->mass_si = r.d();
    o->diameter = r.d();
    o->k_fe = r.d();
    o->k_si = r.d();
    o->kr_fe = r.d();
    o->kr_si = r.d();
    o->sd_fe = r.d();
    o->sd_si = r.d();
    o->n = r.i();
    o->nfe1 = r.i();
    o->nsi1 = r.i();
    o->nfe2 = r.i();
    o->nsi2 = r.i();
    return r.ok ? GI_OK : GI_ERR_FORMAT;
}

extern "C" int gi_write_body_params(const char *path, const gi_body_params *p)
{
    if (!p || !path) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return GI_ERR_IO;
    const struct { const char *name; double v; } reals[] = {
        {"UnitTime", p->unit_time}, {"UnitLength", p->unit_length}, {"UnitMass", p->unit_mass},
        {"MassFe", p->mass_fe},     {"MassSi", p->mass_si},         {"Diameter", p->diameter},
        {"KFe", p->k_fe},           {"KSi", p->k_si},               {"KRFe", p->kr_fe},
        {"KRSi", p->kr_si},         {"SDFe", p->sd_fe},             {"SDSi", p->sd_si}};
    for (const auto &e : reals) std::fprintf(f, "\n %s = %f", e.name, e.v);
    const struct { const char *name; int v; } ints[] = {{"TotalNumberOfElements", p->n},
                                                        {"NFe1", p->nfe1},
                                                        {"NSi1", p->nsi1},
                                                        {"NFe2", p->nfe2},
                                                        {"NSi2", p->nsi2}};
    for (const auto &e : ints) std::fprintf(f, "\n %s = %d", e.name, e.v);
    return std::fclose(f) == 0 ? GI_OK : GI_ERR_IO;
}

extern "C" int gi_read_view_centering(const char *path, float out[6])
{
    if (!out) return GI_ERR_INVALID_ARG;
    std::string t;
    if (int st = open_text(path, t)) return st;
    OrderedReader r(t);
    for (int k = 0; k < 6; ++k) out[k] = r.f();
    return r.ok ? GI_OK : GI_ERR_FORMAT;
}

extern "C" int gi_write_view_centering(const char *path, const float v[6])
{
    if (!v || !path) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return GI_ERR_IO;
    static const char *names[6] = {"InitialCenterOfMassX",   "InitialCenterOfMassY",
                                   "InitialCenterOfMassZ",   "InitialLinearVelocityX",
                                   "InitialLinearVelocityY", "InitialLinearVelocityZ"};
    for (int k = 0; k < 6; ++k) std::fprintf(f, "\n %s = %f\n", names[k], v[k]);
    return std::fclose(f) == 0 ? GI_OK : GI_ERR_IO;
}

// ------------------------------------------------------------------ units --

extern "C" int gi_derive_units(const gi_setup_generating *g, gi_generation_plan *o)
{
    if (!g || !o) return GI_ERR_INVALID_ARG;
    std::memset(o, 0, sizeof *o);
    if (g->frac_fe1 + g->frac_si1 != 1.0 || g->frac_fe2 + g->frac_si2 != 1.0) return GI_ERR_PARAMS;
    if (g->n <= 0) return GI_ERR_BAD_SIZE;
    const double mb1 = kMassOfEarth * g->frac_earth_mass1;
    const double mb2 = kMassOfEarth * g->frac_earth_mass2;
    const double fe1 = g->frac_fe1 * mb1, si1 = g->frac_si1 * mb1;
    const double fe2 = g->frac_fe2 * mb2, si2 = g->frac_si2 * mb2;
    const double fe = fe1 + fe2, si = si1 + si2;
    const double rho = g->density_si / g->density_fe;
    const int nfe = fe != 0.0 ? (int)((double)g->n * rho / (si / fe + rho)) : 0;
    const int nsi = g->n - nfe;
    const int nfe1 = fe != 0.0 ? (int)(nfe * fe1 / fe) : 0;
    const int nsi1 = si != 0.0 ? (int)(nsi * si1 / si) : 0;
    const double mfe = nfe != 0 ? fe / nfe : 0.0;
    const double msi = nsi != 0 ? si / nsi : 0.0;
    double ul, um, ut;
    if (nsi != 0) {
        ul = std::pow((6.0 * msi) / (kPi * g->density_si), 1.0 / 3.0);
        um = msi;
        ut = std::sqrt((6.0 * msi * (double)nsi) / (kUniversalGravity * kPi * g->density_si * si));
    } else if (nfe != 0) {
        ul = std::pow((6.0 * mfe) / (kPi * g->density_fe), 1.0 / 3.0);
        um = mfe;
        ut = std::sqrt((6.0 * mfe * (double)nfe) / (kUniversalGravity * kPi * g->density_fe * fe));
    } else {
        return GI_ERR_PARAMS;
    }
    gi_body_params &b = o->body;
    b.unit_time = ut;
    b.unit_length = ul;
    b.unit_mass = um;
    b.diameter = 1.0;
    if (nsi != 0) {
        b.mass_si = 1.0;
        b.mass_fe = g->density_fe / g->density_si;
    } else {
        b.mass_fe = 1.0;
        b.mass_si = -1.0;  // the reference leaves its initial value
    }
    b.k_fe = g->k_fe * ut * ut * ul / um;
    b.k_si = g->k_si * ut * ut * ul / um;
    b.kr_fe = g->kr_fe;
    b.kr_si = g->kr_si;
    b.sd_fe = g->sd_fe;
    b.sd_si = g->sd_si;
    b.n = g->n;
    b.nfe1 = nfe1;
    b.nsi1 = nsi1;
    b.nfe2 = nfe - nfe1;
    b.nsi2 = nsi - nsi1;
    o->mass_body1 = mb1 / um;
    o->mass_body2 = mb2 / um;
    o->damp_time = g->damp_time * 3600.0 / ut;
    o->damp_rest_time = g->damp_rest_time * 3600.0 / ut;
    o->spin_rest_time = g->spin_rest_time * 3600.0 / ut;
    o->spin1_w = (float)(g->spin1[3] * (ut / 3600.0));
    o->spin2_w = (float)(g->spin2[3] * (ut / 3600.0));
    o->radius_of_earth = kRadiusOfEarth / ul;
    return GI_OK;
}

extern "C" int gi_collision_consts_from_body_params(const gi_body_params *b, double dt,
                                                    gi_force_collision_consts *fc,
                                                    gi_move_collision_consts *mc)
{
    if (!b || !fc || !mc) return GI_ERR_INVALID_ARG;
    if (!counts_ok(*b)) return GI_ERR_BAD_SIZE;
    const double D = b->diameter;
    fc->GMassFeFe = (float)(b->mass_fe * b->mass_fe);  // G = 1
    fc->GMassFeSi = (float)b->mass_fe;                 // G = 1, mSi = 1
    fc->KFeFe = (float)(2.0 * b->k_fe);
    fc->KSiSi = (float)(2.0 * b->k_si);
    fc->KFeSi = (float)(b->k_fe + b->k_si);
    fc->KRFeFe = (float)(2.0 * b->k_fe * b->kr_fe);
    fc->KRSiSi = (float)(2.0 * b->k_si * b->kr_si);
    fc->KRFeSi = (float)(b->k_fe * b->kr_fe + b->k_si * b->kr_si);
    fc->KRMix = (float)(b->sd_fe >= b->sd_si ? b->k_fe + b->k_si * b->kr_si
                                             : b->k_fe * b->kr_fe + b->k_si);
    fc->ShellBreakFe = (float)(D - D * b->sd_fe);
    fc->ShellBreakSi = (float)(D - D * b->sd_si);
    const double s_hi = D - D * (b->sd_fe >= b->sd_si ? b->sd_si : b->sd_fe);
    const double s_lo = D - D * (b->sd_fe >= b->sd_si ? b->sd_fe : b->sd_si);
    fc->ShellBreakFeSi1 = (float)s_hi;
    fc->ShellBreakFeSi2 = (float)s_lo;
    fc->NFe = b->nfe1 + b->nfe2;
    mc->Dt = (float)dt;
    mc->DtOverMassFe = (float)(dt / b->mass_fe);
    mc->DtOverMassSi = (float)(dt / b->mass_si);
    mc->NFe = fc->NFe;
    return GI_OK;
}

extern "C" int gi_separate_consts_from_body_params(const gi_body_params *b, double dt,
                                                   gi_force_separate_consts *fc,
                                                   gi_move_separate_consts *mc)
{
    if (!b || !fc || !mc) return GI_ERR_INVALID_ARG;
    if (!counts_ok(*b)) return GI_ERR_BAD_SIZE;
    gi_force_collision_consts c;
    gi_move_collision_consts m;
    gi_collision_consts_from_body_params(b, dt, &c, &m);
    const double G = 1.0;
    fc->GMassFeFe = (float)(G * b->mass_fe * b->mass_fe);
    fc->GMassFeSi = (float)(G * b->mass_fe * b->mass_si);
    fc->KFeFe = c.KFeFe;
    fc->KSiSi = c.KSiSi;
    fc->KFeSi = c.KFeSi;
    fc->KRFeFe = c.KRFeFe;
    fc->KRSiSi = c.KRSiSi;
    fc->KRFeSi = c.KRFeSi;
    fc->KRMix = c.KRMix;
    fc->ShellBreakFe = c.ShellBreakFe;
    fc->ShellBreakSi = c.ShellBreakSi;
    fc->ShellBreakFeSi1 = c.ShellBreakFeSi1;
    fc->ShellBreakFeSi2 = c.ShellBreakFeSi2;
    fc->boarder1 = b->nfe1;
    fc->boarder2 = b->nfe1 + b->nsi1;
    fc->boarder3 = b->nfe1 + b->nsi1 + b->nfe2;
    mc->Dt = m.Dt;
    mc->DtOverMassFe = m.DtOverMassFe;
    mc->DtOverMassSi = m.DtOverMassSi;
    mc->boarder1 = fc->boarder1;
    mc->boarder2 = fc->boarder2;
    mc->boarder3 = fc->boarder3;
    return GI_OK;
}

// ----------------------------------------------------------- binary files --

extern "C" int gi_write_body_file(const char *path, const float *pos, const float *vel, int n)
{
    if (!path || n < 0 || (n > 0 && (!pos || !vel))) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return GI_ERR_IO;
    bool ok = std::fwrite(&n, sizeof(int), 1, f) == 1;
    ok = ok && std::fwrite(pos, 16, (size_t)n, f) == (size_t)n;
    ok = ok && std::fwrite(vel, 16, (size_t)n, f) == (size_t)n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GI_OK : GI_ERR_IO;
}

extern "C" int gi_read_body_file(const char *path, float *pos, float *vel, int capacity, int *n)
{
    if (!path || !n) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "rb");
    if (!f) return GI_ERR_IO;
    int m = 0;
    if (std::fread(&m, sizeof(int), 1, f) != 1 || m < 0) {
        std::fclose(f);
        return GI_ERR_FORMAT;
    }
    *n = m;
    if (!pos || !vel) {  // count only
        std::fclose(f);
        return GI_OK;
    }
    if (capacity < m) {
        std::fclose(f);
        return GI_ERR_BAD_SIZE;
    }
    bool ok = std::fread(pos, 16, (size_t)m, f) == (size_t)m;
    ok = ok && std::fread(vel, 16, (size_t)m, f) == (size_t)m;
    std::fclose(f);
    return ok ? GI_OK : GI_ERR_FORMAT;
}

extern "C" int gi_frames_append(const char *path, float time, const float *pos, const float *vel,
                                int n)
{
    if (!path || n < 0 || (n > 0 && (!pos || !vel))) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "ab");
    if (!f) return GI_ERR_IO;
    bool ok = std::fwrite(&time, sizeof(float), 1, f) == 1;
    ok = ok && std::fwrite(pos, 16, (size_t)n, f) == (size_t)n;
    ok = ok && std::fwrite(vel, 16, (size_t)n, f) == (size_t)n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GI_OK : GI_ERR_IO;
}

extern "C" int gi_frames_count(const char *path, int n, long long *nframes)
{
    if (!path || n < 0 || !nframes) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "rb");
    if (!f) return GI_ERR_IO;
    std::fseek(f, 0, SEEK_END);
    const long long size = std::ftell(f);
    std::fclose(f);
    const long long frame = 4 + 32LL * n;
    *nframes = size / frame;
    // A partly written last frame would make a resumed run (which seeks one
    // frame back from the end) read a misaligned frame: report it.
    return size % frame == 0 ? GI_OK : GI_ERR_FORMAT;
}

extern "C" int gi_frames_read(const char *path, int n, long long frame, float *time, float *pos,
                              float *vel)
{
    if (!path || n < 0 || !time || (n > 0 && (!pos || !vel))) return GI_ERR_INVALID_ARG;
    long long count = 0;
    if (int st = gi_frames_count(path, n, &count)) return st;
    if (frame < 0) frame = count - 1;
    if (frame < 0 || frame >= count) return GI_ERR_BAD_SIZE;
    FILE *f = std::fopen(path, "rb");
    if (!f) return GI_ERR_IO;
    const long long bytes = 4 + 32LL * n;
    bool ok = std::fseek(f, (long)(frame * bytes), SEEK_SET) == 0;
    ok = ok && std::fread(time, sizeof(float), 1, f) == 1;
    ok = ok && std::fread(pos, 16, (size_t)n, f) == (size_t)n;
    ok = ok && std::fread(vel, 16, (size_t)n, f) == (size_t)n;
    std::fclose(f);
    return ok ? GI_OK : GI_ERR_FORMAT;
}

// ----------------------------------------------------------- body builder --

extern "C" int gi_raw_bodies(unsigned long long seed, const gi_body_params *b, float *pos,
                             float *vel, long long *redraws)
{
    if (!b || (b->n > 0 && (!pos || !vel))) return GI_ERR_INVALID_ARG;
    if (!counts_ok(*b)) return GI_ERR_BAD_SIZE;
    if (!(b->diameter > 0.0)) return GI_ERR_PARAMS;
    gi_host::Rng g(seed);
    const double D = b->diameter;
    const double stretch = 2.0;
    long long total_redraws = 0;
    const long long redraw_limit = 4000LL * (b->n + 1000);
    for (int body = 1; body <= 2; ++body) {
        const int nfe = body == 1 ? b->nfe1 : b->nfe2;
        const int nsi = body == 1 ? b->nsi1 : b->nsi2;
        double volume = ((4.0 / 3.0) * kPi * D * D * D * (double)nfe / 0.68) * stretch;
        const double r1 = cbrt_det(volume / ((4.0 / 3.0) * kPi));
        volume = ((4.0 / 3.0) * kPi * D * D * D * (double)(nfe + nsi) / 0.68) * stretch;
        const double r2 = cbrt_det(volume / ((4.0 / 3.0) * kPi));
        const BodyRanges rg = body_ranges(*b, body);
        for (int group = 0; group < 2; ++group) {
            const int lo = group == 0 ? rg.fe0 : rg.si0, hi = group == 0 ? rg.fe1 : rg.si1;
            const float tag = (float)(2 * (body - 1) + group);
            const float mass = (float)(group == 0 ? b->mass_fe : b->mass_si);
            GroupGrid grid;
            grid.next.assign((size_t)(hi - lo), -1);
            for (int i = lo; i < hi; ++i) {
                float *p = pos + 4 * (size_t)i;
                for (;;) {
                    if (total_redraws > redraw_limit) return GI_ERR_PARAMS;
                    p[0] = (float)(g.uniform() * 2.0 - 1.0);
                    p[1] = (float)(g.uniform() * 2.0 - 1.0);
                    p[2] = (float)(g.uniform() * 2.0 - 1.0);
                    const double mag = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
                    const double u = g.uniform();
                    if (mag == 0.0) continue;  // no direction: draw again
                    const double radius = group == 0 ? u * r1 : u * (r2 - r1) + r1 + D;
                    p[0] = (float)(p[0] * (radius / mag));
                    p[1] = (float)(p[1] * (radius / mag));
                    p[2] = (float)(p[2] * (radius / mag));
                    // closer than D to an earlier element of this group?
                    const int cx = GroupGrid::cell(p[0]), cy = GroupGrid::cell(p[1]),
                              cz = GroupGrid::cell(p[2]);
                    bool clash = false;
                    for (int ox = -1; ox <= 1 && !clash; ++ox)
                        for (int oy = -1; oy <= 1 && !clash; ++oy)
                            for (int oz = -1; oz <= 1 && !clash; ++oz) {
                                auto it = grid.head.find(GroupGrid::key(cx + ox, cy + oy, cz + oz));
                                if (it == grid.head.end()) continue;
                                for (int j = it->second; j >= 0; j = grid.next[j - lo]) {
                                    const float *q = pos + 4 * (size_t)j;
                                    const float dx = p[0] - q[0], dy = p[1] - q[1],
                                                dz = p[2] - q[2];
                                    const double sep = std::sqrt(dx * dx + dy * dy + dz * dz);
                                    if (sep < D) { clash = true; break; }
                                }
                            }
                    if (!clash) {
                        auto ins = grid.head.emplace(GroupGrid::key(cx, cy, cz), i);
                        if (!ins.second) {
                            grid.next[i - lo] = ins.first->second;
                            ins.first->second = i;
                        }
                        break;
                    }
                    ++total_redraws;
                }
                p[3] = tag;
                float *v = vel + 4 * (size_t)i;
                v[0] = v[1] = v[2] = 0.0f;
                v[3] = mass;
            }
        }
    }
    if (redraws) *redraws = total_redraws;
    return GI_OK;
}

extern "C" int gi_spin_body(float *pos, float *vel, const gi_generation_plan *plan, int body,
                            const float axis[3], float w)
{
    if (!pos || !vel || !plan || !axis || (body != 1 && body != 2)) return GI_ERR_INVALID_ARG;
    if (!counts_ok(plan->body)) return GI_ERR_BAD_SIZE;
    float s[3] = {axis[0], axis[1], axis[2]};
    const double mag = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (!(0.0000001 < mag)) return GI_ERR_PARAMS;
    for (int c = 0; c < 3; ++c) s[c] = (float)(s[c] / mag);
    double com[3];
    body_mean(pos, *plan, body, com);
    const BodyRanges r = body_ranges(plan->body, body);
    for (int i = r.fe0; i < r.si1; ++i) {
        const float *p = pos + 4 * (size_t)i;
        float *v = vel + 4 * (size_t)i;
        const double rx = p[0] - com[0], ry = p[1] - com[1], rz = p[2] - com[2];
        const double mag2 = rx * rx + ry * ry + rz * rz;
        const double along = s[0] * rx + s[1] * ry + s[2] * rz;
        // The reference takes sqrt of this difference as is; rounding can make
        // it slightly negative for a body on the axis, which is clamped here.
        const double perp2 = mag2 - along * along;
        const double perp = perp2 > 0.0 ? std::sqrt(perp2) : 0.0;
        const double speed = w * 2.0 * kPi * perp;
        double nx = s[1] * rz - s[2] * ry;
        double ny = -(s[0] * rz - s[2] * rx);
        double nz = s[0] * ry - s[1] * rx;
        const double nm = std::sqrt(nx * nx + ny * ny + nz * nz);
        if (nm != 0.0) {
            nx /= nm;
            ny /= nm;
            nz /= nm;
            v[0] = (float)(v[0] + speed * nx);
            v[1] = (float)(v[1] + speed * ny);
            v[2] = (float)(v[2] + speed * nz);
        }
    }
    return GI_OK;
}

extern "C" int gi_zero_drift(float *pos, float *vel, const gi_generation_plan *plan)
{
    if (!pos || !vel || !plan) return GI_ERR_INVALID_ARG;
    if (!counts_ok(plan->body)) return GI_ERR_BAD_SIZE;
    for (int body = 1; body <= 2; ++body) {
        double c[3], u[3];
        body_mean(pos, *plan, body, c);
        body_mean(vel, *plan, body, u);
        const BodyRanges r = body_ranges(plan->body, body);
        for (int i = r.fe0; i < r.si1; ++i)
            for (int k = 0; k < 3; ++k) {
                pos[4 * (size_t)i + k] = (float)(pos[4 * (size_t)i + k] - c[k]);
                vel[4 * (size_t)i + k] = (float)(vel[4 * (size_t)i + k] - u[k]);
            }
    }
    return GI_OK;
}

extern "C" int gi_write_target_impactor_stats(const char *path, const gi_generation_plan *plan,
                                              const gi_setup_generating *setup, double dt,
                                              const float *pos, const float *vel)
{
    if (!path || !plan || !setup || !pos || !vel) return GI_ERR_INVALID_ARG;
    const gi_body_params &b = plan->body;
    if (!counts_ok(b)) return GI_ERR_BAD_SIZE;
    FILE *f = std::fopen(path, "wb");
    if (!f) return GI_ERR_IO;
    const double lc = b.unit_length, mc = b.unit_mass, vc = b.unit_length / b.unit_time;
    const double amc = (b.unit_mass * b.unit_length * b.unit_length) / b.unit_time;
    std::fprintf(f, "The conversion parameters to take you to and from our units to the real world units follow\n");
    std::fprintf(f, "\n Simulation length unit is %f kilometers", b.unit_length);
    std::fprintf(f, "\n Simulation mass unit is %e kilograms", b.unit_mass);
    std::fprintf(f, "\n Simulation time unit is %f seconds", b.unit_time);
    std::fprintf(f, "\n\n The initail statistics for this run in Simulation units follow\n");
    std::fprintf(f, "\n Diameter of an element: \t\t\tDiameter = %f", b.diameter);
    std::fprintf(f, "\n Gravitational constant: \t\t\tGravity = %f", 1.0);
    std::fprintf(f, "\n The mass of a silicate element: \tMassSi = %f", b.mass_si);
    std::fprintf(f, "\n The mass of an iron element: \t\tMassFe = %f", b.mass_fe);
    std::fprintf(f, "\n\n The push back strength of iron: \tKFe = %f", b.k_fe);
    std::fprintf(f, "\n The push back strength of silicate: \tKSi = %f\n", b.k_si);
    std::fprintf(f, "\n The mass of body one: \tMassOfBody1 = %f", plan->mass_body1);
    std::fprintf(f, "\n The mass of body two: \tMassOfBody2 = %f\n", plan->mass_body2);
    for (int body = 1; body <= 2; ++body) {
        const float *s = body == 1 ? setup->spin1 : setup->spin2;
        const double w = body == 1 ? plan->spin1_w : plan->spin2_w;
        const double m = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
        std::fprintf(f, "\n The initial spin in revolutions per time unit of body %s: (%f, %f, %f, %f)%s",
                     body == 1 ? "one" : "two", s[0] / m, s[1] / m, s[2] / m, w,
                     body == 1 ? "" : "\n");
    }
    const int nfe = b.nfe1 + b.nfe2, nsi = b.nsi1 + b.nsi2;
    std::fprintf(f, "\n Total number of elements: \t\t\t\t\t\tTotalNumberOfElements = %d", b.n);
    std::fprintf(f, "\n Total number of iron elements: \t\t\t\t\tNFe = %d", nfe);
    std::fprintf(f, "\n Total number of silicate elements: \t\t\t\tNSi = %d", nsi);
    std::fprintf(f, "\n Total number of iron elements in body1: \t\t\tNFe1 = %d", b.nfe1);
    std::fprintf(f, "\n Total number of silicate elements in body1: \t\tNSi1 = %d", b.nsi1);
    std::fprintf(f, "\n Total number of iron elements in body2 \t\t\tNFe2: = %d", b.nfe2);
    std::fprintf(f, "\n Total number of silicate elements in body2: \t\tNSi2 = %d\n", b.nsi2);
    std::fprintf(f, "\n Time step in Simulation units: \t\tDt = %f", dt);
    std::fprintf(f, "\n Time step in seconds:\t\t\t\t\tDt = %f", dt * b.unit_time);
    std::fprintf(f, "\n Damp time in Simulation units: \t\tDampTime = %f", plan->damp_time);
    std::fprintf(f, "\n Damp rest time in Simulation units: \tDampRestTime = %f", plan->damp_rest_time);
    std::fprintf(f, "\n Spin rest time in Simulation units: \tSpinRestTime = %f", plan->spin_rest_time);
    std::fprintf(f, "\n\n\n*****************************************************************************************************");
    std::fprintf(f, "\nThe follow are the statistics of the final created bodies in real world units");
    std::fprintf(f, "\n*****************************************************************************************************");
    for (int body = 1; body <= 2; ++body) {
        double c[3], u[3], L[3];
        body_mean(pos, *plan, body, c);
        const double radius = body_radius(pos, *plan, body);
        const double mass = body == 1 ? b.mass_fe * (double)b.nfe1 + b.mass_si * (double)b.nsi1
                                      : b.mass_fe * (double)b.nfe2 + b.mass_si * (double)b.nsi2;
        std::fprintf(f, "\n\n ***** Stats for Body%d *****", body);
        std::fprintf(f, "\n Mass =  %e Kilograms", mass * mc);
        std::fprintf(f, "\n Radius =  %f Kilometers", radius * lc);
        std::fprintf(f, "\n The center of mass = (%f, %f, %f) Kilometers from (0, 0, 0)", c[0] * lc,
                     c[1] * lc, c[2] * lc);
        body_mean(vel, *plan, body, u);
        const double um = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        std::fprintf(f, "\n The average linear velocity = (%f, %f, %f) Kilometers/second", u[0] * vc,
                     u[1] * vc, u[2] * vc);
        std::fprintf(f, "\n The magitude of the avergae linear velocity = %f Kilometers/second", um * vc);
        body_angular_momentum(pos, vel, *plan, body, L);
        const double Lm = std::sqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
        std::fprintf(f, "\n The angular momentum = (%e, %e, %e) Kilograms*kilometers*kilometers/second",
                     L[0] * amc, L[1] * amc, L[2] * amc);
        std::fprintf(f, "\n The magitude of the angular momentum = %e Kilograms*kilometers*kilometers/second",
                     Lm * amc);
    }
    std::fprintf(f, "\n\n");
    return std::fclose(f) == 0 ? GI_OK : GI_ERR_IO;
}

// ------------------------------------------------------------ impact init --

extern "C" int gi_impact_initial_conditions(const gi_body_params *b, const gi_setup_impact_init *s,
                                            const float *pos_in, const float *vel_in,
                                            float *pos_out, float *vel_out)
{
    if (!b || !s || !pos_in || !vel_in || !pos_out || !vel_out) return GI_ERR_INVALID_ARG;
    if (!counts_ok(*b)) return GI_ERR_BAD_SIZE;
    if (!(b->unit_length > 0.0) || !(b->unit_time > 0.0)) return GI_ERR_PARAMS;
    const int n = b->n, n1 = b->nfe1 + b->nsi1;
    // float4 offsets divided / multiplied in double and stored as float
    // (impactInitialization.cu:233-249)
    float dp[2][3], dv[2][3];
    for (int k = 0; k < 3; ++k) {
        dp[0][k] = (float)(s->pos1[k] / b->unit_length);
        dp[1][k] = (float)(s->pos2[k] / b->unit_length);
        dv[0][k] = (float)(s->vel1[k] * (b->unit_time / b->unit_length));
        dv[1][k] = (float)(s->vel2[k] * (b->unit_time / b->unit_length));
    }
    std::vector<float> tp(pos_in, pos_in + 4 * (size_t)n), tv(vel_in, vel_in + 4 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const int body = i < n1 ? 0 : 1;
        for (int k = 0; k < 3; ++k) {
            tp[4 * (size_t)i + k] += dp[body][k];
            tv[4 * (size_t)i + k] += dv[body][k];
        }
    }
    const int seg[4][2] = {{0, b->nfe1}, {n1, n1 + b->nfe2}, {b->nfe1, n1}, {n1 + b->nfe2, n}};
    size_t k = 0;
    for (const auto &sg : seg)
        for (int i = sg[0]; i < sg[1]; ++i, ++k) {
            std::memcpy(pos_out + 4 * k, &tp[4 * (size_t)i], 16);
            std::memcpy(vel_out + 4 * k, &tv[4 * (size_t)i], 16);
        }
    return GI_OK;
}

extern "C" int gi_system_stats_host(const float *pos, const float *vel, int n, int nfe,
                                    double mass_fe, double mass_si, double out[10])
{
    if (!out || n < 0 || nfe < 0 || nfe > n || (n > 0 && (!pos || !vel))) return GI_ERR_INVALID_ARG;
    double M = 0.0;
    for (int i = 0; i < n; ++i) M += i < nfe ? mass_fe : mass_si;
    double c[3] = {0, 0, 0}, u[3] = {0, 0, 0}, L[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
        const double m = i < nfe ? mass_fe : mass_si;
        for (int k = 0; k < 3; ++k) c[k] += pos[4 * (size_t)i + k] * m;
    }
    for (int k = 0; k < 3; ++k) c[k] /= M;
    for (int i = 0; i < n; ++i) {
        const double m = i < nfe ? mass_fe : mass_si;
        for (int k = 0; k < 3; ++k) u[k] += vel[4 * (size_t)i + k] * m;
    }
    for (int k = 0; k < 3; ++k) u[k] /= M;
    for (int i = 0; i < n; ++i) {
        const double m = i < nfe ? mass_fe : mass_si;
        const float *p = pos + 4 * (size_t)i, *v = vel + 4 * (size_t)i;
        const double rx = p[0] - c[0], ry = p[1] - c[1], rz = p[2] - c[2];
        const double vx = v[0] - u[0], vy = v[1] - u[1], vz = v[2] - u[2];
        L[0] += (ry * vz - rz * vy) * m;
        L[1] += -(rx * vz - rz * vx) * m;
        L[2] += (rx * vy - ry * vx) * m;
    }
    out[0] = M;
    for (int k = 0; k < 3; ++k) {
        out[1 + k] = c[k];
        out[4 + k] = u[k];
        out[7 + k] = L[k];
    }
    return GI_OK;
}

extern "C" int gi_write_initial_stats(const char *path, const gi_body_params *b,
                                      const double st[10])
{
    if (!path || !b || !st) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return GI_ERR_IO;
    const double mc = b->unit_mass, lc = b->unit_length, vc = b->unit_length / b->unit_time;
    const double pc = b->unit_mass * b->unit_length * b->unit_length / b->unit_time;
    std::fprintf(f, "\n\n\n*************************************************************************\n\n");
    std::fprintf(f, "\nThe following are the initial stats of the impact\n");
    std::fprintf(f, "\nDistance is measured in Kilometers");
    std::fprintf(f, "\nMass is measured in Kilograms");
    std::fprintf(f, "\nTime is measured in seconds");
    std::fprintf(f, "\nVelocity is measured in Kilometers/second");
    std::fprintf(f, "\nAngular momentun is measured in Kilograms*Kilometers*Kilometers/seconds\n");
    double x = st[1] * lc, y = st[2] * lc, z = st[3] * lc;
    std::fprintf(f, "\nCenter of mass of the entire system \t\t        = (%f, %f, %f)\n", x, y, z);
    std::fprintf(f, "\nTotal mass of the entire system \t= %e\n", st[0] * mc);
    x = st[4] * vc; y = st[5] * vc; z = st[6] * vc;
    std::fprintf(f, "\nLinear velocity of the entire system system \t\t= (%f, %f, %f)", x, y, z);
    std::fprintf(f, "\nMagnitude of the linear velocity of the entire system \t= %f\n",
                 std::sqrt(x * x + y * y + z * z));
    x = st[7] * pc; y = st[8] * pc; z = st[9] * pc;
    std::fprintf(f, "\nAngular momentum of the entire system system \t\t= (%e, %e, %e)", x, y, z);
    std::fprintf(f, "\nMagnitude of the angular momentum of the entire system \t= %e\n",
                 std::sqrt(x * x + y * y + z * z));
    std::fprintf(f, "\n\n*************************************************************************\n\n\n");
    return std::fclose(f) == 0 ? GI_OK : GI_ERR_IO;
}

// ----------------------------------------------------------- final stats --

namespace {

void composition(FILE *f, const char *who, const int c[4])
{
    // c = [Fe body 1, Fe body 2, Si body 1, Si body 2]
    std::fprintf(f, "\n%s iron from body 1 \t\t= %d", who, c[0]);
    std::fprintf(f, "\n%s silicate from body 1 \t= %d", who, c[2]);
    std::fprintf(f, "\n%s iron from body 2 \t\t= %d", who, c[1]);
    std::fprintf(f, "\n%s silicate from body 2 \t= %d", who, c[3]);
    const int b1 = c[0] + c[2], b2 = c[1] + c[3];
    if (b2 == 0) std::fprintf(f, "\nThe %s is only composed of elements from body 1\n", who);
    else if (b1 == 0) std::fprintf(f, "\nThe %s is only composed of elements from body 2\n", who);
    else std::fprintf(f, "\n%s ratio body1/body2 \t\t= %f\n", who, (float)b1 / (float)b2);
}

void spin_lines(FILE *f, const char *what, const char *mag_name, const char *angle_name,
                const double *S, double pc)
{
    const double x = S[7] * pc, y = S[8] * pc, z = S[9] * pc;
    std::fprintf(f, "\nAngular momentum of %s= (%e, %e, %e)", what, x, y, z);
    const double mag = std::sqrt(x * x + y * y + z * z);
    std::fprintf(f, "\nMagnitude of the angular momentum of %s= %e", mag_name, mag);
    const double size = std::sqrt(x * x + y * y + z * z) * std::sqrt(x * x + z * z);
    const double angle = std::acos((x * x + z * z) / size);
    std::fprintf(f, "\nAngle off ecliptic plane of %s= %f\n", angle_name,
                 90.0 - angle * 180.0 / kPi);
}

}  // namespace

extern "C" int gi_write_run_stats(const char *path, const gi_body_params *b, double time,
                                  const gi_earth_moon *em, const double S[4][15])
{
    if (!path || !b || !em || !S) return GI_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return GI_ERR_IO;
    const double tc = b->unit_time, lc = b->unit_length, mc = b->unit_mass;
    const double vc = b->unit_length / b->unit_time;
    const double pc = b->unit_mass * b->unit_length * b->unit_length / b->unit_time;
    const double mE = S[2][0], mM = S[3][0];
    std::fprintf(f, "\n\n\n*************************************************************************\n\n");
    std::fprintf(f, "\nThe following are the final stats of the run when time = %f hours\n",
                 time * tc / 3600.0);
    std::fprintf(f, "\nDistance is measured in Kilometers");
    std::fprintf(f, "\nMass is measured in Kilograms");
    std::fprintf(f, "\nTime is measured in seconds");
    std::fprintf(f, "\nVelocity is measured in Kilometers/second");
    std::fprintf(f, "\nAngular momentun is measured in Kilograms*Kilometers*Kilometers/seconds\n");
    std::fprintf(f, "\nThe mass of Earth \t\t= %e", mE * mc);
    std::fprintf(f, "\nThe mass of Moon \t\t= %e", mM * mc);
    if (mM != 0.0) std::fprintf(f, "\nThe mass ratio Earth/Moon \t= %f\n", mE / mM);
    composition(f, "Moon", em->moon_counts);
    composition(f, "Earth", em->earth_counts);
    spin_lines(f, "the Earth Moon system \t\t", "the system \t", "the system's rotation \t",
               S[1], pc);
    spin_lines(f, "the Earth \t\t\t\t", "the Earth \t\t", "the Earth's rotation \t", S[2], pc);
    spin_lines(f, "the Moon \t\t\t\t", "the Moon \t\t", "the Moon's rotation \t", S[3], pc);
    std::fprintf(f, "\nCenter of mass of the Earth-Moon system \t\t= (%f, %f, %f)", S[1][1] * lc,
                 S[1][2] * lc, S[1][3] * lc);
    std::fprintf(f, "\nCenter of mass of the Earth system \t\t\t= (%f, %f, %f)", S[2][1] * lc,
                 S[2][2] * lc, S[2][3] * lc);
    std::fprintf(f, "\nCenter of mass of the Moon system \t\t\t= (%f, %f, %f)\n", S[3][1] * lc,
                 S[3][2] * lc, S[3][3] * lc);
    std::fprintf(f, "\nLinear Velocity of the Earth-Moon system \t\t= (%f, %f, %f)", S[1][4] * vc,
                 S[1][5] * vc, S[1][6] * vc);
    std::fprintf(f, "\nLinear Velocity of the Earth system \t\t\t= (%f, %f, %f)", S[2][4] * vc,
                 S[2][5] * vc, S[2][6] * vc);
    std::fprintf(f, "\nLinear Velocity of the Moon system \t\t\t= (%f, %f, %f)\n", S[3][4] * vc,
                 S[3][5] * vc, S[3][6] * vc);
    std::fprintf(f, "\n*****Stats of the entire system to check the numerical scheme's validity*****\n");
    std::fprintf(f, "\nCenter of mass of the entire system \t\t        = (%f, %f, %f)\n",
                 S[0][1] * lc, S[0][2] * lc, S[0][3] * lc);
    std::fprintf(f, "\nTotal mass of the entire system \t= %f\n", S[0][0]);
    double x = S[0][4] * vc, y = S[0][5] * vc, z = S[0][6] * vc;
    std::fprintf(f, "\nLinear velocity of the entire system system \t\t= (%f, %f, %f)", x, y, z);
    std::fprintf(f, "\nMagnitude of the linear velocity of the entire system \t= %f\n",
                 std::sqrt(x * x + y * y + z * z));
    x = S[0][7] * pc; y = S[0][8] * pc; z = S[0][9] * pc;
    std::fprintf(f, "\nAngular momentum of the entire system system \t\t= (%e, %e, %e)", x, y, z);
    std::fprintf(f, "\nMagnitude of the angular momentum of the entire system \t= %e\n",
                 std::sqrt(x * x + y * y + z * z));
    std::fprintf(f, "\n\n*************************************************************************\n\n\n");
    return std::fclose(f) == 0 ? GI_OK : GI_ERR_IO;
}
