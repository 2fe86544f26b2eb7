// cfgio.cu - configuration files and checkpoints of the resident state (host code).
//
//   mdg_write_cfg        config_output (src/config.f90:244-301) with the records of write_rigmol,
//                        write_atmol, write_surfmol, write_crystal and write_thermostat
//                        (:484-590): box, type count, per molecule type its name/kind/count and
//                        records, derivatives converted back to 1 fs units, Fortran E15.8 fields
//   mdg_read_cfg         config_input (:174-242) and read_rigmol/atmol/surfmol/crystal/thermostat
//                        (:395-482), then config_init (:55-95: derivatives to time-step units,
//                        sites from the quaternions) and move_shake_init (src/move.f90:394-396:
//                        previous positions of surface and wall atoms equal to the current ones)
//   mdg_checkpoint_*     the resident state's device arrays in binary, with a header that the
//                        loading context must match
// Everything goes through mdg_get_state / mdg_set_state, so the device layout stays private.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"
#include "ctx.h"

namespace mdg {

namespace {

const char* kKind[4] = {"rigmol", "atmol", "surfmol", "crystal"};

// Fortran Ew.d output (w = 15, d = 8): [-]0.dddddddd E[+-]ee, right-justified in 15 columns.
std::string fort_e(double x, bool full) {
    char b[64];
    if (full) {
        snprintf(b, sizeof b, " %24.17E", x);
        return b;
    }
    if (x == 0.0) return "  0.00000000E+00";
    if (!std::isfinite(x)) {
        snprintf(b, sizeof b, " %15s", "NaN");
        return b;
    }
    // x = m 10^e with 0.1 <= |m| < 1 after rounding m to 8 digits
    int e = (int)std::floor(std::log10(std::fabs(x))) + 1;
    double m = x / std::pow(10.0, e);
    double r = std::round(std::fabs(m) * 1e8);
    if (r >= 1e8) {
        r /= 10.0;
        r = std::round(r);
        ++e;
    } else if (r < 1e7) {
        r = std::round(std::fabs(m) * 1e9);
        --e;
    }
    snprintf(b, sizeof b, "%s0.%08lldE%c%02d", x < 0 ? "-" : "", (long long)r, e < 0 ? '-' : '+', std::abs(e));
    char o[64];
    snprintf(o, sizeof o, " %15s", b);
    return o;
}

struct HostState {
    std::vector<double> x[3], xd[4][3], c[5][3], q[4][5], w[5][3], old[3], rs[3];
    mdg_state st{};
    void alloc(int64_t ntota, int64_t nrig, int64_t nold, int64_t nmove) {
        const int64_t nr = std::max<int64_t>(nrig, 1), no = std::max<int64_t>(nold, 1);
        for (int d = 0; d < 3; ++d) {
            x[d].assign(ntota, 0.0);
            old[d].assign(no, 0.0);
            rs[d].assign(std::max<int64_t>(nmove, 1), 0.0);
            for (int k = 0; k < 4; ++k) xd[k][d].assign(ntota, 0.0);
            for (int k = 0; k < 5; ++k) {
                c[k][d].assign(nr, 0.0);
                w[k][d].assign(nr, 0.0);
            }
        }
        for (int cc = 0; cc < 4; ++cc)
            for (int k = 0; k < 5; ++k) q[cc][k].assign(nr, 0.0);
        st.x0 = x[0].data();
        st.y0 = x[1].data();
        st.z0 = x[2].data();
        for (int k = 0; k < 4; ++k) {
            st.xd[k] = xd[k][0].data();
            st.yd[k] = xd[k][1].data();
            st.zd[k] = xd[k][2].data();
        }
        for (int k = 0; k < 5; ++k) {
            st.cx[k] = c[k][0].data();
            st.cy[k] = c[k][1].data();
            st.cz[k] = c[k][2].data();
            st.wx[k] = w[k][0].data();
            st.wy[k] = w[k][1].data();
            st.wz[k] = w[k][2].data();
            for (int cc = 0; cc < 4; ++cc) st.q[cc][k] = q[cc][k].data();
        }
        st.xold = old[0].data();
        st.yold = old[1].data();
        st.zold = old[2].data();
        st.rsx = rs[0].data();
        st.rsy = rs[1].data();
        st.rsz = rs[2].data();
    }
};

// Whitespace-separated records, one per line (Fortran list-directed input reads one record per
// READ statement and ignores the rest of the line).
struct Records {
    std::vector<std::string> lines;
    size_t at = 0;
    bool next(std::vector<std::string>& tok) {
        tok.clear();
        if (at >= lines.size()) return false;
        std::istringstream ss(lines[at++]);
        std::string t;
        while (ss >> t) tok.push_back(t);
        return true;
    }
};

double fnum(const std::string& s) {
    std::string t = s;
    for (char& ch : t)
        if (ch == 'd' || ch == 'D') ch = 'e';
    return std::stod(t);
}

}  // namespace

int write_cfg(Ctx& c, const char* path, const char* const* names, int full) {
    const mdg_sysdesc& s = c.sysc;
    if (!path || !names) return set_err(&c, MDG_E_ARG, "write_cfg: null argument");
    if (!c.resident) return set_err(&c, MDG_E_ARG, "write_cfg: no resident state (mdg_set_state first)");
    HostState h;
    h.alloc(s.ntota, s.nrig, s.ntota - s.nliqa, s.nmove);
    int rc = mdg_get_state(static_cast<mdg_ctx*>(&c), &h.st);
    if (rc) return rc;
    // walls: mdg_get_state returns the moving atoms; frozen positions come from the device
    if (s.nwall > 0) {
        for (int d = 0; d < 3; ++d) {
            double* src = d == 0 ? c.v.x : (d == 1 ? c.v.y : c.v.z);
            MDG_CUDA(cudaMemcpy(h.x[d].data() + s.nmove, src + s.nmove, sizeof(double) * s.nwall, cudaMemcpyDeviceToHost));
        }
    }
    double th[TH_N];
    MDG_CUDA(cudaMemcpy(th, c.d_thermo, sizeof(th), cudaMemcpyDeviceToHost));
    const double dt = s.dt;
    FILE* f = fopen(path, "w");
    if (!f) return set_err(&c, MDG_E_ARG, std::string("write_cfg: cannot open ") + path);
    auto row = [&](std::initializer_list<double> v) {
        for (double x : v) fputs(fort_e(x, full != 0).c_str(), f);
        fputc('\n', f);
    };
    fprintf(f, " # SIMULATION BOX SIZE\n");
    if (full) fprintf(f, " %.17g %.17g %.17g\n\n", s.lx, s.ly, s.lz);
    else fprintf(f, " %14.10f %14.10f %14.10f\n\n", s.lx, s.ly, s.lz);
    fprintf(f, " # NUMBER OF PARTICLE TYPES\n %lld\n\n # PARTICLE COORDINATES\n", (long long)s.ntype);
    int64_t atom = 0, mol = 0;
    for (int64_t it = 0; it < s.ntype; ++it) {
        const int64_t kind = c.h_moltypen[it], nt = c.h_nt[it], ns = c.h_ns[it];
        fprintf(f, " %s %s %lld\n", names[it], kKind[kind & 3], (long long)nt);
        if (kind == 0) {  // rigmol: molecule records
            for (int64_t i = mol; i < mol + nt; ++i) {
                fprintf(f, " %5lld", (long long)(i + 1));
                for (int64_t k = 0; k < ns; ++k) fprintf(f, " %5lld", (long long)c.h_itype[ns * i + k]);
                fputc('\n', f);
                row({h.c[0][0][i], h.c[0][1][i], h.c[0][2][i]});
                for (int k = 1; k < 5; ++k) {
                    const double sc = std::pow(dt, k);
                    row({h.c[k][0][i] / sc, h.c[k][1][i] / sc, h.c[k][2][i] / sc});
                }
                for (int k = 0; k < 5; ++k) row({h.q[0][k][i], h.q[1][k][i], h.q[2][k][i], h.q[3][k][i]});
                for (int k = 0; k < 5; ++k) {
                    const double sc = std::pow(dt, k + 1);
                    row({h.w[k][0][i] / sc, h.w[k][1][i] / sc, h.w[k][2][i] / sc});
                }
            }
            mol += nt;
            atom += nt * ns;
        } else {
            const int64_t n = nt * ns;
            const int64_t t0 = n > 0 ? c.h_itype[atom] - 1 : 0;
            for (int64_t i = atom; i < atom + n; ++i) {
                const long long code = (long long)(c.h_itype[i] - t0);  // site type within the molecule type
                fprintf(f, " %5lld %5lld\n", (long long)(i + 1), code);
                row({h.x[0][i], h.x[1][i], h.x[2][i]});
                if (kind == 1) {
                    for (int k = 0; k < 4; ++k) {
                        const double sc = std::pow(dt, k + 1);
                        row({h.xd[k][0][i] / sc, h.xd[k][1][i] / sc, h.xd[k][2][i] / sc});
                    }
                } else if (kind == 2) {
                    const int64_t o = i - s.nliqa;
                    row({h.x[0][i] + (h.old[0][o] - h.x[0][i]) / dt, h.x[1][i] + (h.old[1][o] - h.x[1][i]) / dt,
                         h.x[2][i] + (h.old[2][o] - h.x[2][i]) / dt});
                }
            }
            atom += n;
        }
        fputc('\n', f);
    }
    fprintf(f, " # THERMOSTAT\n");
    row({th[TH_S], th[TH_S + 1], th[TH_S + 2], th[TH_S + 3], th[TH_S + 4]});
    row({th[TH_RS], th[TH_RS + 1], th[TH_RS + 2], th[TH_RS + 3], th[TH_RS + 4]});
    const bool ok = ferror(f) == 0;
    fclose(f);
    if (!ok) return set_err(&c, MDG_E_ARG, "write_cfg: write failed");
    return MDG_OK;
}

int read_cfg(Ctx& c, const char* path, const char* const* names, const mdg_rigid* body) {
    const mdg_sysdesc& s = c.sysc;
    if (!path || !names || !body) return set_err(&c, MDG_E_ARG, "read_cfg: null argument");
    std::ifstream in(path);
    if (!in) return set_err(&c, MDG_E_ARG, std::string("read_cfg: cannot open ") + path);
    Records r;
    for (std::string line; std::getline(in, line);) r.lines.push_back(line);
    std::vector<std::string> t;
    auto need = [&](size_t n, const char* what) -> bool {
        if (!r.next(t) || t.size() < n) {
            c.err = std::string("read_cfg: bad record (") + what + ")";
            return false;
        }
        return true;
    };
    try {
        if (!need(1, "box header")) return MDG_E_ARG;
        if (!need(3, "box")) return MDG_E_ARG;
        const double lx = fnum(t[0]), ly = fnum(t[1]), lz = fnum(t[2]);
        if (std::fabs(lx - s.lx) > 1e-6 * s.lx || std::fabs(ly - s.ly) > 1e-6 * s.ly || std::fabs(lz - s.lz) > 1e-6 * s.lz)
            return set_err(&c, MDG_E_ARG, "read_cfg: box differs from the context's");
        r.next(t);
        if (!need(1, "types header") || !need(1, "type count")) return MDG_E_ARG;
        if (std::stoll(t[0]) != s.ntype) return set_err(&c, MDG_E_ARG, "config_input(): wrong number of types!");
        r.next(t);
        if (!need(1, "coordinates header")) return MDG_E_ARG;
        HostState h;
        h.alloc(s.ntota, s.nrig, s.ntota - s.nliqa, s.nmove);
        const double dt = s.dt;
        int64_t atom = 0, mol = 0;
        for (int64_t it = 0; it < s.ntype; ++it) {
            if (!need(3, "molecule type")) return MDG_E_ARG;
            const int64_t kind = c.h_moltypen[it], nt = c.h_nt[it], ns = c.h_ns[it];
            if (t[0] != names[it] || t[1] != kKind[kind & 3] || std::stoll(t[2]) != nt)
                return set_err(&c, MDG_E_ARG, "config_input(): Error in configfile!");
            if (kind == 0) {
                for (int64_t j = 0; j < nt; ++j) {
                    if (!need(1, "molecule")) return MDG_E_ARG;
                    const int64_t i = std::stoll(t[0]) - 1;
                    if (i < 0 || i >= s.nrig) return set_err(&c, MDG_E_ARG, "read_cfg: molecule index out of range");
                    for (int k = 0; k < 5; ++k) {
                        if (!need(3, "centre of mass")) return MDG_E_ARG;
                        const double sc = std::pow(dt, k);
                        for (int d = 0; d < 3; ++d) h.c[k][d][i] = fnum(t[d]) * sc;
                    }
                    for (int k = 0; k < 5; ++k) {
                        if (!need(4, "quaternion")) return MDG_E_ARG;
                        for (int cc = 0; cc < 4; ++cc) h.q[cc][k][i] = fnum(t[cc]);
                    }
                    for (int k = 0; k < 5; ++k) {
                        if (!need(3, "angular velocity")) return MDG_E_ARG;
                        const double sc = std::pow(dt, k + 1);
                        for (int d = 0; d < 3; ++d) h.w[k][d][i] = fnum(t[d]) * sc;
                    }
                }
                mol += nt;
                atom += nt * ns;
            } else {
                const int64_t n = nt * ns;
                for (int64_t j = 0; j < n; ++j) {
                    if (!need(2, "atom")) return MDG_E_ARG;
                    const int64_t i = std::stoll(t[0]) - 1;
                    if (i < 0 || i >= s.ntota) return set_err(&c, MDG_E_ARG, "read_cfg: atom index out of range");
                    if (!need(3, "position")) return MDG_E_ARG;
                    const double p[3] = {fnum(t[0]), fnum(t[1]), fnum(t[2])};
                    for (int d = 0; d < 3; ++d) h.x[d][i] = p[d];
                    if (kind == 1) {
                        for (int k = 0; k < 4; ++k) {
                            if (!need(3, "derivative")) return MDG_E_ARG;
                            const double sc = std::pow(dt, k + 1);
                            for (int d = 0; d < 3; ++d) h.xd[k][d][i] = fnum(t[d]) * sc;
                        }
                    } else if (kind == 2) {
                        if (!need(3, "previous position")) return MDG_E_ARG;  // replaced by move_shake_init
                    }
                }
                atom += n;
            }
            r.next(t);  // blank line after the type
        }
        if (!need(1, "thermostat header")) return MDG_E_ARG;
        if (!need(5, "thermostat s")) return MDG_E_ARG;
        for (int k = 0; k < 5; ++k) h.st.s[k] = fnum(t[k]);
        if (!need(5, "thermostat rs")) return MDG_E_ARG;
        for (int k = 0; k < 5; ++k) h.st.rs[k] = fnum(t[k]);
        // config_quatsite (src/config.f90:303-329): sites of the rigid molecules; the H offsets
        // rsx relative to the O (src/move.f90:157-161); rsx of the O stays 0
        for (int64_t i = 0; i < s.nrig; ++i) {
            const double q1 = h.q[0][0][i], q2 = h.q[1][0][i], q3 = h.q[2][0][i], q4 = h.q[3][0][i];
            double a[9];
            a[0] = -q1 * q1 + q2 * q2 - q3 * q3 + q4 * q4;
            a[1] = 2.0 * (q3 * q4 - q1 * q2);
            a[2] = 2.0 * (q2 * q3 + q1 * q4);
            a[3] = -2.0 * (q1 * q2 + q3 * q4);
            a[4] = q1 * q1 - q2 * q2 - q3 * q3 + q4 * q4;
            a[5] = 2.0 * (q2 * q4 - q1 * q3);
            a[6] = 2.0 * (q2 * q3 - q1 * q4);
            a[7] = -2.0 * (q1 * q3 + q4 * q2);
            a[8] = -q1 * q1 - q2 * q2 + q3 * q3 + q4 * q4;
            for (int j = 0; j < 3; ++j) {
                const int64_t ix = 3 * i + j;
                h.x[0][ix] = h.c[0][0][i] + a[0] * body->xbody[j] + a[3] * body->ybody[j] + a[6] * body->zbody[j];
                h.x[1][ix] = h.c[0][1][i] + a[1] * body->xbody[j] + a[4] * body->ybody[j] + a[7] * body->zbody[j];
                h.x[2][ix] = h.c[0][2][i] + a[2] * body->xbody[j] + a[5] * body->ybody[j] + a[8] * body->zbody[j];
            }
            for (int j = 1; j < 3; ++j)
                for (int d = 0; d < 3; ++d) h.rs[d][3 * i + j] = h.x[d][3 * i + j] - h.x[d][3 * i];
        }
        // move_shake_init: previous positions of the surface and wall atoms = current positions
        for (int64_t i = s.nliqa; i < s.ntota; ++i)
            for (int d = 0; d < 3; ++d) h.old[d][i - s.nliqa] = h.x[d][i];
        return mdg_set_state(static_cast<mdg_ctx*>(&c), body, &h.st);
    } catch (const std::exception& e) {
        return set_err(&c, MDG_E_ARG, std::string("read_cfg: ") + e.what());
    }
}

// ---- binary checkpoint ------------------------------------------------------------------------
namespace {
const char kMagic[8] = {'M', 'D', 'G', 'C', 'K', 'P', 'T', '1'};
struct CkHeader {
    char magic[8];
    int64_t ntota, nmove, nrig, nliqa, nit, nregions;
    double dt;
    mdg_rigid body;
};
}  // namespace

int checkpoint_save(Ctx& c, const char* path) {
    if (!path) return set_err(&c, MDG_E_ARG, "checkpoint: null path");
    if (!c.resident) return set_err(&c, MDG_E_ARG, "checkpoint: no resident state");
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    CkHeader hd{};
    std::memcpy(hd.magic, kMagic, 8);
    hd.ntota = c.sysc.ntota;
    hd.nmove = c.sysc.nmove;
    hd.nrig = c.sysc.nrig;
    hd.nliqa = c.sysc.nliqa;
    hd.nit = c.sysc.nit;
    hd.nregions = (int64_t)c.snap_regions.size();
    hd.dt = c.sysc.dt;
    hd.body = c.body;
    FILE* f = fopen(path, "wb");
    if (!f) return set_err(&c, MDG_E_ARG, std::string("checkpoint: cannot open ") + path);
    bool ok = fwrite(&hd, sizeof hd, 1, f) == 1;
    std::vector<char> buf;
    for (auto& rg : c.snap_regions) {
        const int64_t n = (int64_t)rg.second;
        buf.resize(rg.second);
        if (cudaMemcpy(buf.data(), rg.first, rg.second, cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
        ok = ok && fwrite(&n, sizeof n, 1, f) == 1 && fwrite(buf.data(), 1, rg.second, f) == rg.second;
    }
    fclose(f);
    if (!ok) return set_err(&c, MDG_E_CUDA, "checkpoint: write failed");
    return MDG_OK;
}

int checkpoint_load(Ctx& c, const char* path) {
    if (!path) return set_err(&c, MDG_E_ARG, "checkpoint: null path");
    FILE* f = fopen(path, "rb");
    if (!f) return set_err(&c, MDG_E_ARG, std::string("checkpoint: cannot open ") + path);
    CkHeader hd{};
    if (fread(&hd, sizeof hd, 1, f) != 1 || std::memcmp(hd.magic, kMagic, 8) != 0) {
        fclose(f);
        return set_err(&c, MDG_E_ARG, "checkpoint: not a checkpoint file");
    }
    if (hd.ntota != c.sysc.ntota || hd.nmove != c.sysc.nmove || hd.nrig != c.sysc.nrig ||
        hd.nliqa != c.sysc.nliqa || hd.nit != c.sysc.nit || hd.dt != c.sysc.dt) {
        fclose(f);
        return set_err(&c, MDG_E_ARG, "checkpoint: written for a different system");
    }
    cudaSetDevice(c.device);
    int rc = resident_alloc(c);
    if (rc) {
        fclose(f);
        return rc;
    }
    if (hd.nregions != (int64_t)c.snap_regions.size()) {
        fclose(f);
        return set_err(&c, MDG_E_ARG, "checkpoint: layout differs");
    }
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<char> buf;
    for (auto& rg : c.snap_regions) {
        int64_t n = 0;
        if (fread(&n, sizeof n, 1, f) != 1 || n != (int64_t)rg.second) {
            fclose(f);
            return set_err(&c, MDG_E_ARG, "checkpoint: layout differs");
        }
        buf.resize(rg.second);
        if (fread(buf.data(), 1, rg.second, f) != rg.second) {
            fclose(f);
            return set_err(&c, MDG_E_ARG, "checkpoint: truncated");
        }
        MDG_CUDA(cudaMemcpy(rg.first, buf.data(), rg.second, cudaMemcpyHostToDevice));
    }
    fclose(f);
    c.body = hd.body;
    const int one = 1;
    MDG_CUDA(cudaMemcpy(c.v.status + ST_FORCE_RB, &one, sizeof(int), cudaMemcpyHostToDevice));
    c.resident = true;
    drop_graphs(c);
    return MDG_OK;
}

}  // namespace mdg

extern "C" {

int mdg_write_cfg(mdg_ctx* cp, const char* path, const char* const* molnames, int full_precision) {
    if (!cp) return mdg::set_err(nullptr, MDG_E_ARG, "null context");
    cudaSetDevice(cp->device);
    return mdg::write_cfg(*cp, path, molnames, full_precision);
}

int mdg_read_cfg(mdg_ctx* cp, const char* path, const char* const* molnames, const mdg_rigid* body) {
    if (!cp) return mdg::set_err(nullptr, MDG_E_ARG, "null context");
    cudaSetDevice(cp->device);
    return mdg::read_cfg(*cp, path, molnames, body);
}

int mdg_checkpoint_save(mdg_ctx* cp, const char* path) {
    if (!cp) return mdg::set_err(nullptr, MDG_E_ARG, "null context");
    cudaSetDevice(cp->device);
    return mdg::checkpoint_save(*cp, path);
}

int mdg_checkpoint_load(mdg_ctx* cp, const char* path) {
    if (!cp) return mdg::set_err(nullptr, MDG_E_ARG, "null context");
    return mdg::checkpoint_load(*cp, path);
}

}  // extern "C"
