// sysdef.cu - the reference's input files read on the host, for callers written in C or C++.
//
// A Fortran host holds the tables of mdg_sysdesc in its modules after sysdef_input / sysdef_init
// (src/sysdef.f90:83-340, :356-457) and config_input / config_init (src/config.f90:174-242,
// :55-95, config_quatsite :303-329).  These calls build the same tables, the rigid-water body and
// the integrator state from the .fld, .top and .cfg files of a case, so that a C or C++ caller can
// go from the reference's files to mdg_create / mdg_set_state / the drop-in loop without Fortran.
//
// Reading follows Fortran list-directed input: every READ starts on a new record and takes blank-
// or comma-separated items across as many records as it needs; the rest of its last record is
// dropped.  Reals accept D exponents.  The derived quantities use the reference's operations in
// its order (this file is compiled without multiply-add contraction) and its single-precision
// constants, so they equal the Python readers of this package bit for bit.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mdgpu.h"

namespace mdg {
int set_err(struct Ctx* c, int code, const std::string& msg);
}

namespace {

inline double F(float x) { return (double)x; }  // a default-real literal promoted to real*8
const double kPi = F(3.1415926535898f), kA2m = F(1.0e-10f), kFs = F(1.0e-15f), kSixth = F(1.0f / 6.0f);

struct Records {
    std::vector<std::string> lines;
    size_t pos = 0;
    bool ok = true;
    explicit Records(const std::string& text) {
        std::stringstream ss(text);
        std::string l;
        while (std::getline(ss, l)) lines.push_back(l);
    }
    // one READ of n items
    std::vector<std::string> read(size_t n) {
        std::vector<std::string> items;
        while (items.size() < n) {
            if (pos >= lines.size()) {
                ok = false;
                items.resize(n, "0");
                return items;
            }
            std::string l = lines[pos++];
            for (char& ch : l)
                if (ch == ',' || ch == '\t' || ch == '\r') ch = ' ';
            std::stringstream ls(l);
            std::string tok;
            while (ls >> tok) items.push_back(tok);
        }
        items.resize(n);
        return items;
    }
    void skip() { ++pos; }
};

double fnum(const std::string& s) {
    std::string t = s;
    for (char& ch : t)
        if (ch == 'D' || ch == 'd') ch = 'E';
    return std::strtod(t.c_str(), nullptr);
}

int64_t inum(const std::string& s) {
    if (s.find('.') != std::string::npos || s.find('e') != std::string::npos || s.find('E') != std::string::npos)
        return (int64_t)fnum(s);
    return std::strtoll(s.c_str(), nullptr, 10);
}

struct MolType {
    std::string name, kind;
    int64_t nt = 0, ns = 0;
    std::vector<std::string> sitnam;
    std::vector<int64_t> nss;
    std::vector<double> ms, qms;
    std::vector<double> geometry;  // rigmol: ns x 3, row-major
    std::vector<double> lengths;
    std::vector<double> akt, ath;   // surfmol angles: force constant, degrees
    double cx = 0, cy = 0, cz = 0, lw = 0;
    std::vector<double> qshift;
};

struct Vdw {
    int64_t ijt = 0;
    int kind = 0;  // 0 zero, 1 Lennard-Jones, 2 Buckingham
    double p[3] = {0, 0, 0};
};

int kind_code(const std::string& k) {
    if (k == "rigmol") return 0;
    if (k == "atmol") return 1;
    if (k == "surfmol") return 2;
    if (k == "crystal") return 3;
    return -1;
}

bool read_file(const char* path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

}  // namespace

struct mdg_sysdef {
    mdg_sysdesc d{};
    mdg_rigid body{};
    mdg_state st{};
    std::vector<MolType> mts;
    std::vector<Vdw> vdw;
    std::vector<std::string> names;
    std::vector<const char*> name_ptrs;
    // tables behind d
    std::vector<int64_t> moltypen, nt, ns, nst, nconst, nangt, nss_wall, nsi, ijtype, vdwnum, itype, ictype, constra,
        constrb, iatype, ang1, ang2, ang3;
    std::vector<double> eps, sig, aa, rhoi, cc, qs, mi, mii, length, kt, theta;
    // state behind st
    std::vector<double> x0, y0, z0, xd, c, q, w, xold, yold, zold, rsx, rsy, rsz;
};

namespace {

// sysdef_input, the .fld part (src/sysdef.f90:91-171)
bool parse_fld(const std::string& text, mdg_sysdef& S, std::string& err) {
    Records r(text);
    r.read(1);
    const int64_t ntype = inum(r.read(1)[0]);
    if (ntype < 1) {
        err = "fld: no molecule types";
        return false;
    }
    for (int64_t it = 1; it <= ntype; ++it) {
        r.read(1);
        const std::vector<std::string> h = r.read(4);
        if (inum(h[0]) != it) {
            err = "sysdef_input(): wrong molecule number!";
            return false;
        }
        MolType m;
        m.name = h[1];
        m.kind = h[2];
        m.nt = inum(h[3]);
        r.read(1);
        const int64_t nst = inum(r.read(1)[0]);
        for (int64_t k = 0; k < nst; ++k) {
            const std::vector<std::string> a = r.read(2);
            m.sitnam.push_back(a[0]);
            m.nss.push_back(inum(a[1]));
            const std::vector<std::string> b = r.read(2);
            m.ms.push_back(fnum(b[0]));
            m.qms.push_back(fnum(b[1]));
            m.ns += m.nss.back();
        }
        if (m.kind == "rigmol") {
            r.read(1);
            for (int64_t s = 0; s < m.ns; ++s)
                for (const std::string& v : r.read(3)) m.geometry.push_back(fnum(v));
        } else if (m.kind == "atmol") {
        } else if (m.kind == "surfmol") {
            r.read(1);
            const int64_t nc = inum(r.read(1)[0]);
            for (int64_t k = 0; k < nc; ++k) m.lengths.push_back(fnum(r.read(1)[0]));
            r.read(1);
            const int64_t na = inum(r.read(1)[0]);
            for (int64_t k = 0; k < na; ++k) {
                const std::vector<std::string> a = r.read(2);
                m.akt.push_back(fnum(a[0]));
                m.ath.push_back(fnum(a[1]));
            }
        } else if (m.kind == "crystal") {
            m.ns = inum(r.read(1)[0]);
            const std::vector<std::string> cxyz = r.read(3);
            m.cx = fnum(cxyz[0]);
            m.cy = fnum(cxyz[1]);
            m.cz = fnum(cxyz[2]);
            m.lw = fnum(r.read(1)[0]);
            const int64_t nshift = inum(r.read(1)[0]);
            for (int64_t k = 0; k < nshift; ++k) m.qshift.push_back(fnum(r.read(1)[0]));
        } else {
            err = "sysdef_input(): Unknown moltype!";
            return false;
        }
        S.mts.push_back(m);
    }
    r.read(1);
    int64_t ntx = 0;
    for (const MolType& m : S.mts) ntx += (int64_t)m.nss.size();
    for (int64_t k = 0; k < ntx * (ntx + 1) / 2; ++k) {
        Vdw v;
        v.ijt = inum(r.read(1)[0]);
        r.read(3);
        r.read(3);
        const std::string kind = r.read(1)[0];
        if (kind == "zero") {
            v.kind = 0;
        } else if (kind == "12-6") {  // A/r^12 - B/r^6 as Lennard-Jones (src/sysdef.f90:155-160)
            const std::vector<std::string> a = r.read(2);
            const double s = fnum(a[0]), e = fnum(a[1]);
            v.kind = 1;
            v.p[0] = std::pow(s / e, kSixth);
            v.p[1] = std::pow(e, 2.0) / (4.0 * s);
        } else if (kind == "LeJo") {
            const std::vector<std::string> a = r.read(2);
            v.kind = 1;
            v.p[0] = fnum(a[0]);
            v.p[1] = fnum(a[1]);
        } else if (kind == "Buck") {
            const std::vector<std::string> a = r.read(3);
            v.kind = 2;
            for (int j = 0; j < 3; ++j) v.p[j] = fnum(a[j]);
        } else {
            err = "sysdef_input(): Unknown type of interaction!";
            return false;
        }
        if (v.ijt < 1 || v.ijt > ntx * (ntx + 1) / 2) {
            err = "sysdef_input(): pair type out of range";
            return false;
        }
        S.vdw.push_back(v);
    }
    if (!r.ok) {
        err = "fld: unexpected end of file";
        return false;
    }
    return true;
}

// sysdef_input, the .top part (src/sysdef.f90:174-219)
bool parse_top(const std::string& text, mdg_sysdef& S, std::string& err) {
    Records r(text);
    r.read(1);
    for (size_t it = 0; it < S.mts.size(); ++it) {
        const MolType& m = S.mts[it];
        const std::vector<std::string> h = r.read(4);
        if (inum(h[0]) != (int64_t)it + 1 || h[1] != m.name || h[2] != m.kind || inum(h[3]) != m.nt) {
            err = "sysdef_input(): Error in topofile!";
            return false;
        }
        if (m.kind == "rigmol") {
            if (inum(r.read(2)[1]) != m.ns) {
                err = "sysdef_input(): Error in topofile (sites)!";
                return false;
            }
        } else if (m.kind == "atmol") {
            r.read(1);
        } else if (m.kind == "surfmol") {
            int64_t nsx = inum(r.read(2)[1]);
            if (nsx != (int64_t)m.lengths.size() || nsx > MDG_SMX) {
                err = "sysdef_input(): Error in topofile (nconst)!";
                return false;
            }
            for (int64_t k = 0; k < m.nt; ++k) {
                for (int64_t s = 0; s < MDG_SMX; ++s) {
                    if (s < nsx) {
                        const std::vector<std::string> a = r.read(2);
                        S.constra.push_back(inum(a[0]));
                        S.constrb.push_back(inum(a[1]));
                    } else {
                        S.constra.push_back(0);
                        S.constrb.push_back(0);
                    }
                }
                S.ictype.push_back((int64_t)it + 1);
            }
            nsx = inum(r.read(2)[1]);
            if (nsx != (int64_t)m.akt.size() || nsx > MDG_SMX) {
                err = "sysdef_input(): Error in topofile (nangt)!";
                return false;
            }
            if (nsx > 0)
                for (int64_t k = 0; k < m.nt; ++k) {
                    for (int64_t s = 0; s < MDG_SMX; ++s) {
                        if (s < nsx) {
                            const std::vector<std::string> a = r.read(3);
                            S.ang1.push_back(inum(a[0]));
                            S.ang2.push_back(inum(a[1]));
                            S.ang3.push_back(inum(a[2]));
                        } else {
                            S.ang1.push_back(0);
                            S.ang2.push_back(0);
                            S.ang3.push_back(0);
                        }
                    }
                    S.iatype.push_back((int64_t)it + 1);
                }
        }
    }
    if (!r.ok) {
        err = "top: unexpected end of file";
        return false;
    }
    return true;
}

// sysdef_init (src/sysdef.f90:299-452): counts, pair tables, per-atom tables, rigid body
bool derive(mdg_sysdef& S, double lx, double ly, double lz, double dt, std::string& err) {
    mdg_sysdesc& d = S.d;
    const std::vector<MolType>& mts = S.mts;
    const int64_t ntype = (int64_t)mts.size();
    int64_t nrtype = 0, nltype = 0, nstype = 0, nwtype = 0;
    for (int64_t it = 1; it <= ntype; ++it) {
        const int k = kind_code(mts[it - 1].kind);
        S.moltypen.push_back(k);
        if (k == 0) nrtype = nltype = it;
        if (k == 1) nltype = it;
        if (k == 2) nstype = it;
        if (k == 3) nwtype = it;
        S.nt.push_back(mts[it - 1].nt);
        S.ns.push_back(mts[it - 1].ns);
        S.nst.push_back((int64_t)mts[it - 1].nss.size());
        S.nconst.push_back((int64_t)mts[it - 1].lengths.size());
        S.nangt.push_back((int64_t)mts[it - 1].akt.size());
    }
    if (nwtype != ntype) {
        err = "the crystal must be the last molecule type";
        return false;
    }
    if (S.nt[nwtype - 1] > 1) {
        err = "sysdef_init(): wrong number of crystals";
        return false;
    }
    d.ntype = ntype;
    d.nrig = d.nriga = d.nliqa = d.nsurf = 0;
    for (int64_t it = 0; it < nrtype; ++it) {
        d.nrig += S.nt[it];
        d.nriga += S.ns[it] * S.nt[it];
    }
    for (int64_t it = 0; it < nltype; ++it) d.nliqa += S.ns[it] * S.nt[it];
    for (int64_t it = nltype; it < nstype; ++it) d.nsurf += S.ns[it] * S.nt[it];
    d.nmove = d.nliqa + d.nsurf;
    d.nwall = S.ns[nwtype - 1] * S.nt[nwtype - 1];
    d.ngogo = d.nmove;
    d.ntota = d.nmove + d.nwall;
    d.nit = 0;
    for (int64_t v : S.nst) d.nit += v;
    d.nijt = d.nit * (d.nit + 1) / 2;
    d.nltype = nltype;
    d.ncons = (int64_t)S.ictype.size();
    d.nang = (int64_t)S.iatype.size();
    const MolType& crys = mts[nwtype - 1];
    const int64_t nstw = std::max<int64_t>(2, (int64_t)crys.nss.size());
    for (int64_t k = 0; k < nstw; ++k) S.nss_wall.push_back(k < (int64_t)crys.nss.size() ? crys.nss[k] : 0);
    d.lx = lx;
    d.ly = ly;
    d.lz = lz;
    d.cx = crys.cx;
    d.cy = crys.cy;
    d.cz = crys.cz;
    d.lw = crys.lw;
    d.dt = dt;
    // pair tables (src/sysdef.f90:143-169, :321-335, :362-374)
    const int64_t nit = d.nit, nijt = d.nijt;
    S.ijtype.assign(nit * nit, 0);
    int64_t ijt = 0;
    for (int64_t it = 0; it < nit; ++it)
        for (int64_t jt = it; jt < nit; ++jt) {
            ++ijt;
            S.ijtype[it + nit * jt] = ijt;
            S.ijtype[jt + nit * it] = ijt;
        }
    S.vdwnum.assign(nijt, -1);
    S.eps.assign(nijt, 0.0);
    S.sig.assign(nijt, 0.0);
    S.aa.assign(nijt, 0.0);
    S.rhoi.assign(nijt, 0.0);
    S.cc.assign(nijt, 0.0);
    for (const Vdw& v : S.vdw) {
        const int64_t k = v.ijt - 1;
        S.vdwnum[k] = v.kind;
        if (v.kind == 1) {
            S.sig[k] = v.p[0];
            S.eps[k] = v.p[1];
        } else if (v.kind == 2) {
            S.aa[k] = v.p[0];
            S.rhoi[k] = v.p[1];
            S.cc[k] = v.p[2];
        }
    }
    for (int64_t k = 0; k < nijt; ++k) {
        S.eps[k] = 4.0 * S.eps[k];
        S.sig[k] = std::pow(S.sig[k], 6.0);
        S.rhoi[k] = S.rhoi[k] != 0.0 ? 1.0 / S.rhoi[k] : 0.0;
    }
    // units (src/sysdef.f90:376-379) and per-atom tables (:381-425)
    const double vu = kA2m / (dt * kFs);
    std::vector<std::vector<double>> msi(ntype);
    for (int64_t it = 0; it < ntype; ++it)
        for (double m : mts[it].ms) msi[it].push_back(m * std::pow(vu, 2.0) / 1000.0);
    S.itype.assign(d.ntota, 0);
    S.qs.assign(d.ntota, 0.0);
    S.mi.assign(d.ntota, 0.0);
    S.nsi.assign(nit, 0);
    int64_t i = 0, jjt = 0;
    for (int64_t it = 0; it < std::max(nltype, nstype); ++it) {
        const MolType& m = mts[it];
        for (int64_t mol = 0; mol < m.nt; ++mol) {
            for (size_t ist = 0; ist < m.nss.size(); ++ist) {
                const int64_t iit = jjt + (int64_t)ist + 1;
                S.nsi[iit - 1] = S.moltypen[it] == 0 ? (ist == 0 ? m.ns : 0) : 1;
                for (int64_t a = 0; a < m.nss[ist]; ++a) {
                    if (i >= d.nmove) {
                        err = "sysdef_init(): i /= nmove !";
                        return false;
                    }
                    S.itype[i] = iit;
                    S.mi[i] = msi[it][ist];
                    S.qs[i] = m.qms[ist];
                    ++i;
                }
            }
        }
        jjt += (int64_t)m.nss.size();
    }
    if (i != d.nmove) {
        err = "sysdef_init(): i /= nmove !";
        return false;
    }
    S.mii.assign(d.ntota, 0.0);
    for (int64_t a = 0; a < d.nmove; ++a) S.mii[a] = 1.0 / S.mi[a];
    // constraint lengths, bend constants and angles (src/sysdef.f90:376), ntype x MDG_SMX column-major
    S.length.assign(ntype * MDG_SMX, 0.0);
    S.kt.assign(ntype * MDG_SMX, 0.0);
    S.theta.assign(ntype * MDG_SMX, 0.0);
    for (int64_t it = 0; it < ntype; ++it) {
        for (size_t s = 0; s < mts[it].lengths.size() && s < (size_t)MDG_SMX; ++s) S.length[it + ntype * s] = mts[it].lengths[s];
        for (size_t s = 0; s < mts[it].akt.size() && s < (size_t)MDG_SMX; ++s) {
            S.kt[it + ntype * s] = mts[it].akt[s];
            S.theta[it + ntype * s] = mts[it].ath[s] * kPi / 180.0;
        }
    }
    if (S.constra.empty()) S.constra.assign(MDG_SMX, 0), S.constrb.assign(MDG_SMX, 0), S.ictype.assign(1, 0);
    if (S.ang1.empty()) S.ang1.assign(MDG_SMX, 0), S.ang2.assign(MDG_SMX, 0), S.ang3.assign(MDG_SMX, 0), S.iatype.assign(1, 0);
    // rigid water geometry (src/sysdef.f90:427-452)
    mdg_rigid& b = S.body;
    std::memset(&b, 0, sizeof(b));
    b.temper = -1.0;
    if (mts[0].kind == "rigmol") {
        const MolType& m = mts[0];
        const int64_t nsw = std::min<int64_t>(m.ns, MDG_SMX);
        std::vector<double> g(m.geometry);
        double msum = 0.0;
        for (int64_t s = 0; s < nsw; ++s) msum += S.mi[s];
        for (int dd = 0; dd < 3; ++dd) {
            double gm = 0.0;
            for (int64_t s = 0; s < nsw; ++s) gm += g[3 * s + dd] * S.mi[s];
            gm = gm / msum;
            for (int64_t s = 0; s < nsw; ++s) g[3 * s + dd] = g[3 * s + dd] - gm;
        }
        b.inxx = b.inyy = b.inzz = 0.0;
        for (int64_t s = 0; s < nsw; ++s) {
            const double gx = g[3 * s], gy = g[3 * s + 1], gz = g[3 * s + 2];
            b.inxx += S.mi[s] * (gy * gy + gz * gz);
            b.inyy += S.mi[s] * (gz * gz + gx * gx);
            b.inzz += S.mi[s] * (gx * gx + gy * gy);
            b.xbody[s] = gx;
            b.ybody[s] = gy;
            b.zbody[s] = gz;
        }
        double mw = 0.0;
        for (size_t k = 0; k < m.nss.size(); ++k) mw += (double)m.nss[k] * msi[0][k];
        b.mw = mw;
    }
    return true;
}

// config_input (src/config.f90:174-242) into the state, crystal sites (src/config.f90:460-471 with
// the type remap of src/sysdef.f90:406-419), then config_init (src/config.f90:55-95)
bool parse_cfg(const std::string& text, mdg_sysdef& S, double dt, std::string& err, double& lx, double& ly,
               double& lz, std::vector<int64_t>& wtype, std::vector<double>& wpos, bool size_only) {
    Records r(text);
    r.read(1);
    const std::vector<std::string> box = r.read(3);
    lx = fnum(box[0]);
    ly = fnum(box[1]);
    lz = fnum(box[2]);
    if (size_only) return r.ok;
    r.skip();
    r.read(1);
    if (inum(r.read(1)[0]) != (int64_t)S.mts.size()) {
        err = "config_input(): wrong number of types!";
        return false;
    }
    r.skip();
    r.read(1);
    const mdg_sysdesc& d = S.d;
    const int64_t nt = d.ntota, nr = d.nrig;
    wtype.assign(d.nwall, 0);
    wpos.assign(3 * d.nwall, 0.0);
    for (const MolType& m : S.mts) {
        const std::vector<std::string> h = r.read(3);
        if (h[0] != m.name || h[1] != m.kind || inum(h[2]) != m.nt) {
            err = "config_input(): Error in configfile!";
            return false;
        }
        if (m.kind == "rigmol") {
            for (int64_t mol = 0; mol < m.nt; ++mol) {
                const int64_t i = inum(r.read(1 + m.ns)[0]) - 1;
                if (i < 0 || i >= nr) {
                    err = "config_input(): molecule index out of range";
                    return false;
                }
                for (int k = 0; k < 5; ++k) {
                    const std::vector<std::string> v = r.read(3);
                    for (int dd = 0; dd < 3; ++dd) S.c[((size_t)k * 3 + dd) * nr + i] = fnum(v[dd]);
                }
                for (int k = 0; k < 5; ++k) {
                    const std::vector<std::string> v = r.read(4);
                    for (int cc = 0; cc < 4; ++cc) S.q[((size_t)cc * 5 + k) * nr + i] = fnum(v[cc]);
                }
                for (int k = 0; k < 5; ++k) {
                    const std::vector<std::string> v = r.read(3);
                    for (int dd = 0; dd < 3; ++dd) S.w[((size_t)k * 3 + dd) * nr + i] = fnum(v[dd]);
                }
            }
        } else if (m.kind == "atmol") {
            for (int64_t a = 0; a < m.nt * m.ns; ++a) {
                const int64_t i = inum(r.read(2)[0]) - 1;
                if (i < 0 || i >= nt) {
                    err = "config_input(): atom index out of range";
                    return false;
                }
                const std::vector<std::string> p = r.read(3);
                S.x0[i] = fnum(p[0]);
                S.y0[i] = fnum(p[1]);
                S.z0[i] = fnum(p[2]);
                for (int k = 0; k < 4; ++k) {
                    const std::vector<std::string> v = r.read(3);
                    for (int dd = 0; dd < 3; ++dd) S.xd[((size_t)k * 3 + dd) * nt + i] = fnum(v[dd]);
                }
            }
        } else if (m.kind == "surfmol") {
            for (int64_t a = 0; a < m.nt * m.ns; ++a) {
                const int64_t i = inum(r.read(2)[0]) - 1;
                if (i < 0 || i >= nt) {
                    err = "config_input(): atom index out of range";
                    return false;
                }
                const std::vector<std::string> p = r.read(3), o = r.read(3);
                const double x = fnum(p[0]), y = fnum(p[1]), z = fnum(p[2]);
                S.x0[i] = x;
                S.y0[i] = y;
                S.z0[i] = z;
                S.xold[i] = x + (fnum(o[0]) - x) * dt;
                S.yold[i] = y + (fnum(o[1]) - y) * dt;
                S.zold[i] = z + (fnum(o[2]) - z) * dt;
            }
        } else if (m.kind == "crystal") {
            for (int64_t a = 0; a < m.nt * m.ns; ++a) {
                const std::vector<std::string> h2 = r.read(2);
                const int64_t k = inum(h2[0]) - 1 - d.nmove;
                if (k < 0 || k >= d.nwall) {
                    err = "config_input(): wall index out of range";
                    return false;
                }
                wtype[k] = inum(h2[1]);
                const std::vector<std::string> p = r.read(3);
                for (int dd = 0; dd < 3; ++dd) wpos[3 * k + dd] = fnum(p[dd]);
            }
        }
        r.skip();
    }
    r.read(1);
    const std::vector<std::string> s5 = r.read(5), r5 = r.read(5);
    for (int k = 0; k < 5; ++k) {
        S.st.s[k] = fnum(s5[k]);
        S.st.rs[k] = fnum(r5[k]);
    }
    if (!r.ok) {
        err = "cfg: unexpected end of file";
        return false;
    }
    return true;
}

}  // namespace

extern "C" {

int mdg_sysdef_load(const char* fld_path, const char* top_path, const char* cfg_path, double dt,
                    mdg_sysdef** out) {
    if (!fld_path || !top_path || !cfg_path || !out || !(dt > 0.0))
        return mdg::set_err(nullptr, MDG_E_ARG, "sysdef_load: null argument or dt <= 0");
    *out = nullptr;
    std::string ftxt, ttxt, ctxt, err;
    if (!read_file(fld_path, ftxt)) return mdg::set_err(nullptr, MDG_E_ARG, std::string("cannot read ") + fld_path);
    if (!read_file(top_path, ttxt)) return mdg::set_err(nullptr, MDG_E_ARG, std::string("cannot read ") + top_path);
    if (!read_file(cfg_path, ctxt)) return mdg::set_err(nullptr, MDG_E_ARG, std::string("cannot read ") + cfg_path);
    mdg_sysdef* S = new (std::nothrow) mdg_sysdef();
    if (!S) return mdg::set_err(nullptr, MDG_E_ARG, "sysdef_load: out of memory");
    double lx = 0, ly = 0, lz = 0;
    std::vector<int64_t> wtype;
    std::vector<double> wpos;
    bool ok = parse_fld(ftxt, *S, err) && parse_top(ttxt, *S, err) &&
              parse_cfg(ctxt, *S, dt, err, lx, ly, lz, wtype, wpos, true) && derive(*S, lx, ly, lz, dt, err);
    if (ok) {
        const mdg_sysdesc& d = S->d;
        const size_t nt = (size_t)d.ntota, nr = (size_t)d.nrig, nm = (size_t)d.nmove;
        S->x0.assign(nt, 0.0);
        S->y0.assign(nt, 0.0);
        S->z0.assign(nt, 0.0);
        S->xd.assign(12 * nt, 0.0);
        S->c.assign(15 * nr, 0.0);
        S->q.assign(20 * nr, 0.0);
        S->w.assign(15 * nr, 0.0);
        S->xold.assign(nt, 0.0);
        S->yold.assign(nt, 0.0);
        S->zold.assign(nt, 0.0);
        S->rsx.assign(nm, 0.0);
        S->rsy.assign(nm, 0.0);
        S->rsz.assign(nm, 0.0);
        ok = parse_cfg(ctxt, *S, dt, err, lx, ly, lz, wtype, wpos, false);
    }
    if (!ok) {
        delete S;
        return mdg::set_err(nullptr, MDG_E_ARG, err);
    }
    mdg_sysdesc& d = S->d;
    const int64_t nt = d.ntota, nr = d.nrig, nmv = d.nmove;
    // crystal sites: charge by type code, negative codes are the charge shifts (src/config.f90:460-471)
    const MolType& crys = S->mts[d.ntype - 1];
    const int64_t jjt_wall = d.nit - (int64_t)crys.nss.size();
    for (int64_t k = 0; k < d.nwall; ++k) {
        const int64_t i = nmv + k;
        int64_t is = wtype[k];
        if (is > 0 && is <= (int64_t)crys.qms.size()) {
            S->qs[i] = crys.qms[is - 1];
        } else if (is < 0 && -is <= (int64_t)crys.qshift.size()) {
            S->qs[i] = crys.qshift[-is - 1];
            is = (crys.nss.empty() || -is <= crys.nss[0]) ? 1 : 2;
        } else {
            delete S;
            return mdg::set_err(nullptr, MDG_E_ARG, "config_input(): crystal site type out of range");
        }
        S->itype[i] = jjt_wall + is;
        S->x0[i] = wpos[3 * k];
        S->y0[i] = wpos[3 * k + 1];
        S->z0[i] = wpos[3 * k + 2];
    }
    // config_init (src/config.f90:55-95): derivatives to time-step units, then the sites
    for (int k = 0; k < 4; ++k) {
        const double f = std::pow(dt, (double)(k + 1));
        for (int64_t i = 0; i < 3 * nt; ++i) S->xd[(size_t)k * 3 * nt + i] *= f;
        for (int64_t i = 0; i < 3 * nr; ++i) S->c[(size_t)(k + 1) * 3 * nr + i] *= f;
    }
    for (int k = 0; k < 5; ++k) {
        const double f = std::pow(dt, (double)(k + 1));
        for (int64_t i = 0; i < 3 * nr; ++i) S->w[(size_t)k * 3 * nr + i] *= f;
    }
    const mdg_rigid& b = S->body;
    for (int64_t i = 0; i < nr; ++i) {  // config_quatsite (src/config.f90:303-329)
        const double q1 = S->q[(0 * 5 + 0) * nr + i], q2 = S->q[(1 * 5 + 0) * nr + i], q3 = S->q[(2 * 5 + 0) * nr + i],
                     q4 = S->q[(3 * 5 + 0) * nr + i];
        const double a00 = -q1 * q1 + q2 * q2 - q3 * q3 + q4 * q4, a01 = 2.0 * (q3 * q4 - q1 * q2),
                     a02 = 2.0 * (q2 * q3 + q1 * q4), a10 = -2.0 * (q1 * q2 + q3 * q4),
                     a11 = q1 * q1 - q2 * q2 - q3 * q3 + q4 * q4, a12 = 2.0 * (q2 * q4 - q1 * q3),
                     a20 = 2.0 * (q2 * q3 - q1 * q4), a21 = -2.0 * (q1 * q3 + q4 * q2),
                     a22 = -q1 * q1 - q2 * q2 + q3 * q3 + q4 * q4;
        const double cx = S->c[0 * nr + i], cy = S->c[1 * nr + i], cz = S->c[2 * nr + i];
        for (int j = 0; j < 3; ++j) {
            const int64_t a = 3 * i + j;
            S->x0[a] = cx + a00 * b.xbody[j] + a10 * b.ybody[j] + a20 * b.zbody[j];
            S->y0[a] = cy + a01 * b.xbody[j] + a11 * b.ybody[j] + a21 * b.zbody[j];
            S->z0[a] = cz + a02 * b.xbody[j] + a12 * b.ybody[j] + a22 * b.zbody[j];
        }
    }
    // the description's pointers
    d.moltypen = S->moltypen.data();
    d.nt = S->nt.data();
    d.ns = S->ns.data();
    d.nst = S->nst.data();
    d.nconst = S->nconst.data();
    d.nangt = S->nangt.data();
    d.nss_wall = S->nss_wall.data();
    d.nsi = S->nsi.data();
    d.ijtype = S->ijtype.data();
    d.vdwnum = S->vdwnum.data();
    d.eps = S->eps.data();
    d.sig = S->sig.data();
    d.aa = S->aa.data();
    d.rhoi = S->rhoi.data();
    d.cc = S->cc.data();
    d.itype = S->itype.data();
    d.qs = S->qs.data();
    d.mi = S->mi.data();
    d.mii = S->mii.data();
    d.ictype = S->ictype.data();
    d.constra = S->constra.data();
    d.constrb = S->constrb.data();
    d.length = S->length.data();
    d.iatype = S->iatype.data();
    d.ang1 = S->ang1.data();
    d.ang2 = S->ang2.data();
    d.ang3 = S->ang3.data();
    d.kt = S->kt.data();
    d.theta = S->theta.data();
    // the state's pointers: xd[k] x-component of derivative k+1 (3 x ntota per k), c[k] (3 x nrig),
    // q[c][k] (5 x nrig per component), w[k]
    mdg_state& st = S->st;
    st.x0 = S->x0.data();
    st.y0 = S->y0.data();
    st.z0 = S->z0.data();
    for (int k = 0; k < 4; ++k) {
        st.xd[k] = S->xd.data() + ((size_t)k * 3 + 0) * nt;
        st.yd[k] = S->xd.data() + ((size_t)k * 3 + 1) * nt;
        st.zd[k] = S->xd.data() + ((size_t)k * 3 + 2) * nt;
    }
    for (int k = 0; k < 5; ++k) {
        st.cx[k] = S->c.data() + ((size_t)k * 3 + 0) * nr;
        st.cy[k] = S->c.data() + ((size_t)k * 3 + 1) * nr;
        st.cz[k] = S->c.data() + ((size_t)k * 3 + 2) * nr;
        st.wx[k] = S->w.data() + ((size_t)k * 3 + 0) * nr;
        st.wy[k] = S->w.data() + ((size_t)k * 3 + 1) * nr;
        st.wz[k] = S->w.data() + ((size_t)k * 3 + 2) * nr;
        for (int cc = 0; cc < 4; ++cc) st.q[cc][k] = S->q.data() + ((size_t)cc * 5 + k) * nr;
    }
    st.xold = S->xold.data() + d.nliqa;
    st.yold = S->yold.data() + d.nliqa;
    st.zold = S->zold.data() + d.nliqa;
    st.rsx = S->rsx.data();
    st.rsy = S->rsy.data();
    st.rsz = S->rsz.data();
    for (const MolType& m : S->mts) S->names.push_back(m.name);
    for (const std::string& n : S->names) S->name_ptrs.push_back(n.c_str());
    *out = S;
    return MDG_OK;
}

const mdg_sysdesc* mdg_sysdef_desc(const mdg_sysdef* sd) { return sd ? &sd->d : nullptr; }
const mdg_rigid* mdg_sysdef_rigid(const mdg_sysdef* sd) { return sd ? &sd->body : nullptr; }
mdg_state* mdg_sysdef_state(mdg_sysdef* sd) { return sd ? &sd->st : nullptr; }
const char* const* mdg_sysdef_molnames(const mdg_sysdef* sd) { return sd ? sd->name_ptrs.data() : nullptr; }
void mdg_sysdef_free(mdg_sysdef* sd) { delete sd; }

}  // extern "C"
