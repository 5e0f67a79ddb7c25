// Input/output surface of FDFK2D and the whole program on the GPU.
//
//   fdfk_input_read     - the input folder: inpar file (src/Input.f90:3-73), FD model, source,
//                         receivers, FK models (src/Input.f90:75-186, 227-284), Vp/Vs SU models
//                         and the material array c (src/Input.f90:288-408)
//   fdfk_backazimuths   - compute_backazimuth_grids (src/coord_transform.f90:1-61, with
//                         src/define_rotation_matrix.f90 and src/calc_backazimuth.f90)
//   fdfk_stable_dt      - check_stability (src/Submain.f90:118-164)
//   fdfk_write_su       - the SU trace files written by src/FDFK2D.f90:547-561
//   fdfk_run            - program FDFK2D (src/FDFK2D.f90:1-157, simulate_wavefield :159-580)
//                         with the time loop, FK background and sampling on the GPU
#include "fdfk_gb300.h"
#include "fdfk_session.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <string>
#include <vector>

using namespace fdfk;

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kDeg2Rad = kPi / 180.0;
constexpr double kRad2Deg = 180.0 / kPi;

// ---------------------------------------------------------------- list-directed text input

// Records of a text file with the Fortran list-directed value separators (blanks, commas)
// turned into a token stream per record.
struct Records {
    std::vector<std::string> lines;
    size_t next = 0;
    bool open(const std::string& path)
    {
        std::ifstream f(path);
        if (!f) return false;
        std::string l;
        while (std::getline(f, l)) {
            if (!l.empty() && l.back() == '\r') l.pop_back();
            lines.push_back(l);
        }
        return true;
    }
    bool skip()
    {
        if (next >= lines.size()) return false;
        ++next;
        return true;
    }
    // One list-directed read of n values starting at the next record (values may continue on
    // the following records; values past n on the last record used are ignored; '/' ends it).
    bool read(size_t n, std::vector<std::string>& out)
    {
        out.clear();
        while (out.size() < n) {
            if (next >= lines.size()) return false;
            const std::string& l = lines[next++];
            size_t i = 0;
            bool slash = false;
            while (i < l.size() && out.size() < n) {
                while (i < l.size() && (l[i] == ' ' || l[i] == '\t' || l[i] == ',')) ++i;
                if (i >= l.size()) break;
                if (l[i] == '/') { slash = true; break; }
                std::string tok;
                if (l[i] == '\'' || l[i] == '"') {
                    const char q = l[i++];
                    while (i < l.size() && l[i] != q) tok += l[i++];
                    ++i;
                } else {
                    while (i < l.size() && l[i] != ' ' && l[i] != '\t' && l[i] != ',' && l[i] != '/') tok += l[i++];
                }
                out.push_back(tok);
            }
            if (slash) break;
        }
        return out.size() == n;
    }
};

bool to_double(std::string t, double& v)
{
    for (char& ch : t)
        if (ch == 'd' || ch == 'D') ch = 'e';
    char* end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return end && end != t.c_str() && *end == '\0';
}
bool to_float(const std::string& t, float& v)
{
    double d;
    if (!to_double(t, d)) return false;
    v = (float)d;
    return true;
}
bool to_int(const std::string& t, int& v)
{
    char* end = nullptr;
    const long x = std::strtol(t.c_str(), &end, 10);
    if (!end || end == t.c_str() || *end != '\0') return false;
    v = (int)x;
    return true;
}
bool to_logical(const std::string& t, int& v)
{
    size_t i = 0;
    while (i < t.size() && t[i] == '.') ++i;
    if (i >= t.size()) return false;
    const char ch = (char)std::tolower((unsigned char)t[i]);
    if (ch != 't' && ch != 'f') return false;
    v = ch == 't' ? 1 : 0;
    return true;
}

int fail(const std::string& m) { return set_error(FDFK_EINVAL, m); }

std::string join(const std::string& dir, const std::string& f)
{
    if (dir.empty()) return f;
    return dir + "/" + f;
}

// Fortran NINT: nearest integer, halves away from zero.
long nint(double x) { return (long)std::lround(x); }

// ---------------------------------------------------------------- geodesy (spherical Earth)

// First column of the reference's inverse rotation (src/define_rotation_matrix.f90): the
// geocentric direction of the local x axis of the profile (y = z = 0 for every grid column).
void profile_axis(double lat_org, double lon_org, double az_org, double col[3])
{
    const double az = az_org * kDeg2Rad, lat = lat_org * kDeg2Rad, lon = lon_org * kDeg2Rad;
    const double st = std::sin(lat), ct = std::cos(lat), sp = std::sin(lon), cp = std::cos(lon);
    const double sa = std::sin(az), ca = std::cos(az);
    col[0] = -sa * sp + ca * st * cp;
    col[1] = sa * cp + ca * st * cp;
    col[2] = -ca * ct;
}

constexpr double kEarthR = 6371.e3;                 // single-precision constant of the reference
constexpr double kFlattening = 1.0 / 298.257;

void geogr2cart(double lat, double lon, double& x, double& y, double& z)
{
    const double col = (90.0 - lat) * kDeg2Rad, lo = lon * kDeg2Rad;
    x = kEarthR * std::sin(col) * std::cos(lo);
    y = kEarthR * std::sin(col) * std::sin(lo);
    z = kEarthR * std::cos(col);
}

void cart2geogr(double x, double y, double z, double& lat, double& lon)
{
    const double r = std::hypot(x, y);
    if (r < 1e-6) {
        lat = z > 0.0 ? 90.0 : -90.0;
        lon = 0.0;
        return;
    }
    lat = std::atan2(z, r) * kRad2Deg;
    lon = std::atan2(y, x) * kRad2Deg;
    if (std::fabs(lat) < 1e-9) lat = 0.0;
    if (std::fabs(lon) < 1e-9) lon = 0.0;
}

// Back-azimuth (degrees) at the station of the event, on the flattened sphere of the reference.
double backaz(double evla, double evlo, double stla, double stlo)
{
    const double coeff = (1.0 - kFlattening) * (1.0 - kFlattening);
    const double scola = 0.5 * kPi - std::atan(coeff * std::tan(stla * kDeg2Rad));
    const double ecola = 0.5 * kPi - std::atan(coeff * std::tan(evla * kDeg2Rad));
    const double slon = stlo * kDeg2Rad, elon = evlo * kDeg2Rad;
    const double c = std::cos(scola);
    const double d = std::sin(slon), e = -std::cos(slon);
    const double g = -c * e, h = c * d, k = -std::sin(scola);
    const double aa = std::sin(ecola) * std::cos(elon), bb = std::sin(ecola) * std::sin(elon), cc = std::cos(ecola);
    const double rhs1 = (aa - d) * (aa - d) + (bb - e) * (bb - e) + cc * cc - 2.0;
    const double rhs2 = (aa - g) * (aa - g) + (bb - h) * (bb - h) + (cc - k) * (cc - k) - 2.0;
    double dbaz = std::atan2(rhs1, rhs2);
    if (dbaz < 0.0) dbaz += 2.0 * kPi;
    double baz = dbaz * kRad2Deg;
    if (std::fabs(baz - 360.0) < 1e-5) baz = 0.0;
    return baz;
}

// ---------------------------------------------------------------- SU files

bool read_su_traces(const std::string& path, int ntr, int ns, float* dst, int comp, int ncomp, std::string& err)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<float> tr(ns);
    char head[240];
    for (int t = 0; t < ntr; ++t) {
        if (!f.read(head, 240) || !f.read(reinterpret_cast<char*>(tr.data()), (std::streamsize)ns * 4)) {
            err = path + ": expected " + std::to_string(ntr) + " traces of " + std::to_string(ns) + " samples";
            return false;
        }
        for (int s = 0; s < ns; ++s) dst[(size_t)ncomp * ((size_t)s + (size_t)ns * t) + comp] = tr[s];
    }
    return true;
}

}  // namespace

extern "C" {

int fdfk_write_su(const char* path, int ntr, int ns, const float* data, int head58, int head59)
{
    if (!path || !data || ntr < 0 || ns < 0) return fail("fdfk_write_su: bad argument");
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) return fail(std::string("cannot write ") + path);
    int16_t head[120];
    std::memset(head, 0, sizeof(head));
    head[57] = (int16_t)head58;
    head[58] = (int16_t)head59;
    for (int t = 0; t < ntr; ++t) {
        f.write(reinterpret_cast<const char*>(head), sizeof(head));
        f.write(reinterpret_cast<const char*>(data + (size_t)ns * t), (std::streamsize)ns * 4);
    }
    if (!f) return fail(std::string("write failed: ") + path);
    return FDFK_OK;
}

int fdfk_backazimuths(double lat_org, double lon_org, double az_org, double evla, double evlo, int n,
                      const float* coordx, double* bazs)
{
    if (!coordx || !bazs || n < 0) return fail("fdfk_backazimuths: bad argument");
    double col[3];
    profile_axis(lat_org, lon_org, az_org, col);
    double xo, yo, zo;
    geogr2cart(lat_org, lon_org, xo, yo, zo);
    for (int i = 0; i < n; ++i) {
        const double X = (double)coordx[i];
        const double x = col[0] * X + xo, y = col[1] * X + yo, z = col[2] * X + zo;
        double stla, stlo;
        cart2geogr(x, y, z, stla, stlo);
        bazs[i] = backaz(evla, evlo, stla, stlo) * kDeg2Rad - az_org * kDeg2Rad;
    }
    return FDFK_OK;
}

int fdfk_stable_dt(int norder, int nx, int nz, int npml, float dx, float dz, const float* c, double* dt_stable)
{
    if (!c || !dt_stable || norder < 1 || norder > 8) return fail("fdfk_stable_dt: bad argument");
    // column norder of fd_coef2 (src/Submain.f90:1202-1245): collocated second-derivative weights
    double sum_abs = 0.0, sum = 0.0;
    for (int j = 1; j <= norder; ++j) {
        double t1 = 1.0, t2 = 1.0, t3 = 1.0;
        for (int k = 1; k <= j - 1; ++k) {
            t1 *= (double)(k * k);
            t2 *= (double)(j * j) - (double)(k * k);
        }
        for (int k = j + 1; k <= norder; ++k) {
            t1 *= (double)(k * k);
            t3 *= (double)(k * k) - (double)(j * j);
        }
        t1 *= (j % 2 == 1) ? 1.0 : -1.0;
        t2 *= (double)(j * j);
        const double cj = t1 / t2 / t3;
        sum_abs += std::fabs(cj);
        sum += cj;
    }
    // check_stability (src/Submain.f90:118-164), single precision as there
    const float h = std::max(dx, dz);
    const float cx = (h / dx) * (h / dx), cz = (h / dz) * (h / dz);
    const float cfl = std::sqrt((float)(2.0 / ((double)(cx + cz) * (sum_abs + sum))));
    const size_t ncell = (size_t)(nz + npml) * (nx + 2 * npml);
    float vmax = 0.f;
    for (size_t i = 0; i < ncell; ++i) vmax = std::max(vmax, std::sqrt((c[3 * i + 1] + 2.0f * c[3 * i + 2]) / c[3 * i]));
    *dt_stable = (double)(cfl * h / vmax);
    return FDFK_OK;
}

int fdfk_input_read(const char* inpath, const char* inparfile, int write_model_copies, fdfk_input* in)
{
    if (!inpath || !inparfile || !in) return fail("fdfk_input_read: NULL argument");
    std::memset(in, 0, sizeof(*in));
    const std::string dir = inpath;
    Records inpar;
    const std::string finpar = join(dir, inparfile);
    if (!inpar.open(finpar)) return fail("cannot open " + finpar);
    std::vector<std::string> v, names;
    for (int i = 0; i < 7; ++i) {
        if (!inpar.read(1, v)) return fail(finpar + ": expected 7 file names");
        names.push_back(v[0]);
    }

    // FD model (src/Input.f90:113-134)
    Records fd;
    if (!fd.open(join(dir, names[0]))) return fail("cannot open " + join(dir, names[0]));
    int fdorder = 0;
    float xn = 0.f, zn = 0.f;
    double dt = 0.0;
    bool ok = fd.skip() && fd.read(1, v) && to_int(v[0], fdorder) && fd.skip() && fd.read(7, v) &&
              to_float(v[0], in->x0) && to_float(v[1], xn) && to_float(v[2], in->z0) && to_float(v[3], zn) &&
              to_float(v[4], in->dx) && to_float(v[5], in->dz) && to_double(v[6], dt);
    in->dt = dt;
    ok = ok && fd.skip() && fd.read(4, v) && to_float(v[0], in->tmax) && to_float(v[1], in->tstp) &&
         to_int(v[2], in->npml) && to_logical(v[3], in->is_PML_top);
    ok = ok && fd.skip() && fd.read(3, v) && to_double(v[0], in->lat_org) && to_double(v[1], in->lon_org) &&
         to_double(v[2], in->az_org);
    ok = ok && fd.skip() && fd.read(2, v) && to_logical(v[0], in->outsnap) && to_int(v[1], in->nstep);
    if (!ok) return fail(join(dir, names[0]) + ": malformed FD model file");
    in->norder = fdorder / 2;
    if (2 * in->norder > in->npml + 1) in->norder = (in->npml + 1) / 2;
    in->nx = (int)nint((double)((xn - in->x0) / in->dx)) + 1;
    in->nz = (int)nint((double)((zn - in->z0) / in->dz)) + 1;
    in->izt = in->is_PML_top ? 1 - in->npml : 1;

    // Source (src/Input.f90:137-148): rayp in s/deg, to s/m
    Records src;
    if (!src.open(join(dir, names[1]))) return fail("cannot open " + join(dir, names[1]));
    ok = src.skip() && src.read(3, v) && to_float(v[0], in->f0) && to_float(v[1], in->ds) &&
         to_logical(v[2], in->src_type) && src.skip() && src.read(3, v) && to_double(v[0], in->rayp) &&
         to_double(v[1], in->evla) && to_double(v[2], in->evlo);
    if (!ok) return fail(join(dir, names[1]) + ": malformed source file");
    in->rayp = in->rayp * 180.0 / (kPi * 6371.e3);

    // Receivers (src/Input.f90:151-157, 227-249)
    Records rcv;
    if (!rcv.open(join(dir, names[2]))) return fail("cannot open " + join(dir, names[2]));
    if (!(rcv.skip() && rcv.read(1, v) && to_int(v[0], in->nrcv) && in->nrcv > 0 && rcv.skip()))
        return fail(join(dir, names[2]) + ": malformed receiver file");
    in->rx = (float*)std::calloc(in->nrcv, sizeof(float));
    in->rz = (float*)std::calloc(in->nrcv, sizeof(float));
    if (!in->rx || !in->rz) return set_error(FDFK_ENOMEM, "host allocation failed");
    const float xmax = in->x0 + (in->nx - 1) * in->dx, zmax = in->z0 + (in->nz - 1) * in->dz;
    for (int r = 0; r < in->nrcv; ++r) {
        if (!(rcv.read(2, v) && to_float(v[0], in->rx[r]) && to_float(v[1], in->rz[r])))
            return fail(join(dir, names[2]) + ": expected " + std::to_string(in->nrcv) + " receivers");
        if (in->rx[r] < in->x0 || in->rx[r] > xmax || in->rz[r] < in->z0 || in->rz[r] > zmax)
            return fail("receiver " + std::to_string(r + 1) + " lies outside the model");
    }

    // FK models (src/Input.f90:160-175, 252-284): vp, vs, z_top per layer; rho from vp
    auto read_fk = [&](const std::string& fn, int& nl, float*& m) -> int {
        Records fk;
        if (!fk.open(join(dir, fn))) return fail("cannot open " + join(dir, fn));
        if (!(fk.skip() && fk.read(1, v) && to_int(v[0], nl) && nl > 0 && fk.skip()))
            return fail(join(dir, fn) + ": malformed FK model file");
        m = (float*)std::calloc(4 * (size_t)nl, sizeof(float));
        if (!m) return set_error(FDFK_ENOMEM, "host allocation failed");
        for (int l = 0; l < nl; ++l) {
            float vp, vs, zt;
            if (!(fk.read(3, v) && to_float(v[0], vp) && to_float(v[1], vs) && to_float(v[2], zt)))
                return fail(join(dir, fn) + ": expected " + std::to_string(nl) + " layers");
            m[4 * l] = zt;
            m[4 * l + 1] = vp;
            m[4 * l + 2] = vs;
            m[4 * l + 3] = (vp + 980.0f) / 2.760f;
        }
        return FDFK_OK;
    };
    int rc = read_fk(names[3], in->nlayer_left, in->fk_left);
    if (rc) return rc;
    if ((rc = read_fk(names[4], in->nlayer_right, in->fk_right))) return rc;
    float dmax = 0.f;
    for (int r = 1; r < 4; ++r)
        dmax = std::max(dmax, std::fabs(in->fk_left[4 * (in->nlayer_left - 1) + r] -
                                        in->fk_right[4 * (in->nlayer_right - 1) + r]));
    if (dmax > 1e-6f) return fail("The bottom half-space must be identical !");

    // Vp, Vs SU models: nx + 2 npml traces of nz + npml - izt + 1 samples (src/Input.f90:288-367)
    const int NX = in->nx + 2 * in->npml, NZ = in->nz + in->npml - in->izt + 1;
    in->c = (float*)std::calloc(3 * (size_t)NX * NZ, sizeof(float));
    if (!in->c) return set_error(FDFK_ENOMEM, "host allocation failed");
    std::string err;
    if (!read_su_traces(join(dir, names[5]), NX, NZ, in->c, 1, 3, err) ||
        !read_su_traces(join(dir, names[6]), NX, NZ, in->c, 2, 3, err))
        return fail(err);
    // the model without its absorbing frame, next to the input models (src/Input.f90:311-321, 346-356)
    if (write_model_copies) {
        for (int comp = 1; comp <= 2; ++comp) {
            std::vector<float> v((size_t)in->nx * in->nz);
            for (int x = 0; x < in->nx; ++x)
                for (int z = 0; z < in->nz; ++z)
                    v[(size_t)z + (size_t)in->nz * x] =
                        in->c[3 * ((size_t)(z + 1 - in->izt) + (size_t)NZ * (x + in->npml)) + comp];
            const std::string src = comp == 1 ? names[5] : names[6];
            const std::string base = src.size() > 3 ? src.substr(0, src.size() - 3) : src;
            const int wr = fdfk_write_su(join(dir, base + "_without_pml.su").c_str(), in->nx, in->nz, v.data(), in->nz, 1000);
            if (wr) return wr;
        }
    }
    // rho from vp, then (rho, lambda, mu) (src/Input.f90:386-405)
    bool neg = false;
    for (size_t i = 0; i < (size_t)NX * NZ; ++i) {
        const float vp = in->c[3 * i + 1], vs = in->c[3 * i + 2];
        neg |= vp < 0.f || vs < 0.f;
        const float rho = (vp + 980.0f) / 2.760f;
        in->c[3 * i] = rho;
        in->c[3 * i + 1] = rho * (vp * vp - 2.0f * vs * vs);
        in->c[3 * i + 2] = rho * vs * vs;
    }
    in->negative_velocity = neg ? 1 : 0;
    return FDFK_OK;
}

void fdfk_input_free(fdfk_input* in)
{
    if (!in) return;
    std::free(in->rx); std::free(in->rz); std::free(in->fk_left); std::free(in->fk_right); std::free(in->c);
    in->rx = in->rz = in->fk_left = in->fk_right = in->c = nullptr;
}

int fdfk_run(const char* inpath, const char* inparfile, const char* outpath, const char* fsis, int write_model_copies)
{
    fdfk_input in;
    int rc = fdfk_input_read(inpath, inparfile, write_model_copies, &in);
    if (rc) {
        fdfk_input_free(&in);
        return rc;
    }
    struct Guard {
        fdfk_input* in;
        fdfk_session* s = nullptr;
        ~Guard()
        {
            fdfk_session_destroy(s);
            fdfk_input_free(in);
        }
    } g{&in};
    const std::string dir = inpath, out = outpath ? outpath : ".", name = fsis && *fsis ? fsis : "seis";
    // rows izt..nz+npml (izt = 1 - npml with the absorbing layer on top)
    const int NX = in.nx + 2 * in.npml, NZ = in.nz + in.npml - in.izt + 1;

    // stability (src/Submain.f90:118-164, every cell of c) and the absorbing-layer constants
    // (src/FDFK2D.f90:407-421)
    double dt_stable = 0.0;
    if ((rc = fdfk_stable_dt(in.norder, in.nx, NZ - in.npml, in.npml, in.dx, in.dz, in.c, &dt_stable))) return rc;
    if (in.dt > dt_stable)
        return fail("The dt is too large to stablize the simulation ! The stable dt = " + std::to_string(dt_stable) +
                    " is recommended");
    float vpml = 0.f;
    for (size_t i = 0; i < (size_t)NX * NZ; ++i)
        vpml = std::max(vpml, std::sqrt((in.c[3 * i + 1] + 2.0f * in.c[3 * i + 2]) / in.c[3 * i]));

    // time axis and sampling (src/FDFK2D.f90:311-317)
    const int nt = (int)nint((double)in.tmax / in.dt);
    float tstp = in.tstp < in.dt ? (float)in.dt : in.tstp;
    const int nstp = (int)nint((double)tstp / in.dt);
    const int nsis = nt / nstp;
    tstp = (float)(nstp * in.dt);

    // back-azimuths of the grid columns (src/FDFK2D.f90:380-402); the reference asks whether to
    // continue when the profile is more than 30 degrees off the back-azimuth: here it warns and goes on
    std::vector<float> coordx(NX);
    for (int ix = 1 - in.npml; ix <= in.nx + in.npml; ++ix) coordx[ix - 1 + in.npml] = in.x0 + (float)(ix - 1) * in.dx;
    std::vector<double> bazs(NX);
    if ((rc = fdfk_backazimuths(in.lat_org, in.lon_org, in.az_org, in.evla, in.evlo, NX, coordx.data(), bazs.data())))
        return rc;
    double sum = 0.0;
    for (double b : bazs) sum += b;
    if (std::fabs(std::cos(sum / (NX + 1))) < 0.5 * std::sqrt(3.0))
        std::fprintf(stderr, "WARNING: the angle between the profile and the back-azimuth exceeds 30 degrees; "
                             "a 2-D simulation of the teleseismic wavefield is inaccurate\n");

    fdfk_params p{};
    p.norder = in.norder; p.nx = in.nx; p.nz = in.nz; p.npml = in.npml; p.is_PML_top = in.is_PML_top ? 1 : 0;
    p.npower = 2;
    p.nbd = 2 * in.norder - 1; p.nt = nt; p.dx = in.dx; p.dz = in.dz; p.dt = in.dt; p.vpml = vpml; p.R0 = 1e-3;
    if ((rc = fdfk_session_create(&p, in.c, &g.s))) return rc;
    double rayp = in.rayp;
    if (std::fabs(rayp) < 1e-9) rayp = rayp < 0.0 ? -1e-9 : 1e-9;   // src/FDFK2D.f90:428
    fdfk_fk_params fk{};
    fk.nx = in.nx; fk.nz = in.nz; fk.npml = in.npml; fk.izt = in.izt; fk.nbd = p.nbd; fk.nt = nt; fk.src_type = in.src_type;
    fk.x0 = in.x0; fk.z0 = in.z0; fk.dx = in.dx; fk.dz = in.dz; fk.dt = in.dt; fk.ds = in.ds; fk.f0 = in.f0;
    fk.rayp = rayp;
    if ((rc = fdfk_session_fk_background(g.s, &fk, bazs.data(), in.nlayer_left, in.fk_left, in.nlayer_right,
                                         in.fk_right)) ||
        (rc = fdfk_session_set_receivers(g.s, in.nrcv, in.rx, in.rz, in.x0, in.z0, nstp, nsis)))
        return rc;

    // the time loop, with snapshots of level 2 every nstep steps (src/FDFK2D.f90:465-532)
    if (in.outsnap && in.nstep > 0) {
        std::error_code ec;
        std::filesystem::create_directories(join(out, "snapshots"), ec);
        if (ec) return fail("cannot create " + join(out, "snapshots") + ": " + ec.message());
        std::vector<float> sx((size_t)in.nz * in.nx), sz((size_t)in.nz * in.nx);
        for (int it = 0; it <= nt;) {
            const int next = std::min(nt + 1, (it / in.nstep + 1) * in.nstep);
            if ((rc = fdfk_session_advance(g.s, next - it))) return rc;
            it = next;
            if (it <= nt) {
                if ((rc = fdfk_session_snapshot(g.s, sx.data(), sz.data()))) return rc;
                char fn[64];
                std::snprintf(fn, sizeof(fn), "snapshots/%05dux.su", it);
                if ((rc = fdfk_write_su(join(out, fn).c_str(), in.nx, in.nz, sx.data(), in.nz, (int)in.dz))) return rc;
                std::snprintf(fn, sizeof(fn), "snapshots/%05duz.su", it);
                if ((rc = fdfk_write_su(join(out, fn).c_str(), in.nx, in.nz, sz.data(), in.nz, (int)in.dz))) return rc;
            }
        }
    } else if ((rc = fdfk_session_advance(g.s, nt + 1))) {
        return rc;
    }
    std::vector<float> seisx((size_t)(nsis + 1) * in.nrcv), seisz(seisx.size());
    if ((rc = fdfk_session_download_seismograms(g.s, seisx.data(), seisz.data()))) return rc;

    // radial component along the back-azimuth of each receiver (src/FDFK2D.f90:537-543), SU output
    std::vector<double> rb(in.nrcv);
    if ((rc = fdfk_backazimuths(in.lat_org, in.lon_org, in.az_org, in.evla, in.evlo, in.nrcv, in.rx, rb.data())))
        return rc;
    for (int r = 0; r < in.nrcv; ++r)
        for (int s = 0; s <= nsis; ++s) {
            float& v = seisx[(size_t)s + (size_t)(nsis + 1) * r];
            v = (float)((double)v * std::cos(rb[r]));
        }
    const int h59 = (int)(int32_t)(tstp * 1e6f);
    if ((rc = fdfk_write_su(join(out, name + "x.su").c_str(), in.nrcv, nsis + 1, seisx.data(), nsis + 1, h59)) ||
        (rc = fdfk_write_su(join(out, name + "z.su").c_str(), in.nrcv, nsis + 1, seisz.data(), nsis + 1, h59)))
        return rc;
    return FDFK_OK;
}

}  // extern "C"
