// scene_io.cpp — the reference's scene files, read on the host: a config.xml
// (SimFramework > simulator, read by BaseSimulator::readSimulatorFromConfigFile,
// Simulator/BaseSimulator.cpp:4-65, and PdIpcSimulator::addModelFromConfigFile /
// addStaticModelFromConfigFile / readExtraAttributeFromConfigFile,
// Simulator/PD-IPC/PdIpcSimulator.h:462-642), each object's <name>/<name>.obj,
// its tetgen <name>.node/.ele pair (volumetric_mesh="tet"), and its
// fixed_points.txt (PdIpcModel::readFixedInfo, PdIpcModel.h:56-77).
//
// Model placement follows BaseModel: with origin (default on) the points move
// so the surface box centre is at the origin, with uniform (default on) they
// are divided by the box's largest extent (BaseModel::init, placeOrigin,
// BaseSurfaceMesh::uniform, Model/BaseModel.cpp:21-66,
// Model/TriangleMesh/BaseSurfaceMesh.cpp:384-402); then <scale> about the
// surface box centre, <translation>, and <rotation> (Z*Y*X Euler angles in
// degrees about the box centre; BaseModel.cpp:411-471).  The tet points move
// with the surface.  Arithmetic is FP64 here (the reference's qeal is float).
// The cached boundary.dat / patchInfo.dat are not read: the library computes
// the same topology (checked against those caches by the known-answer tests).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/pdipc.h"

namespace {

// ---------------- a small XML reader (elements, attributes, text) ----------------
struct XNode {
    std::string name, text;
    std::vector<std::pair<std::string, std::string>> attrs;  // in document order
    std::vector<std::unique_ptr<XNode>> kids;
    const XNode* child(const std::string& n) const {
        for (auto& k : kids)
            if (k->name == n) return k.get();
        return nullptr;
    }
};

struct XParser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit XParser(const std::string& src) : s(src) {}
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }
    bool skip_misc() {  // declarations, comments, doctype
        for (;;) {
            ws();
            if (s.compare(i, 4, "<!--") == 0) {
                size_t e = s.find("-->", i + 4);
                if (e == std::string::npos) return false;
                i = e + 3;
            } else if (s.compare(i, 2, "<?") == 0 || s.compare(i, 2, "<!") == 0) {
                size_t e = s.find('>', i);
                if (e == std::string::npos) return false;
                i = e + 1;
            } else {
                return true;
            }
        }
    }
    std::unique_ptr<XNode> element() {
        if (!skip_misc() || i >= s.size() || s[i] != '<') {
            err = "expected an element";
            return nullptr;
        }
        ++i;
        auto n = std::make_unique<XNode>();
        while (i < s.size() && !std::isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') n->name += s[i++];
        for (;;) {
            ws();
            if (i >= s.size()) { err = "unterminated tag"; return nullptr; }
            if (s[i] == '/') {
                if (s.compare(i, 2, "/>") != 0) { err = "bad tag end"; return nullptr; }
                i += 2;
                return n;
            }
            if (s[i] == '>') { ++i; break; }
            std::string an;
            while (i < s.size() && s[i] != '=' && !std::isspace((unsigned char)s[i])) an += s[i++];
            ws();
            if (i >= s.size() || s[i] != '=') { err = "attribute without value"; return nullptr; }
            ++i;
            ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) { err = "unquoted attribute"; return nullptr; }
            const char q = s[i++];
            size_t e = s.find(q, i);
            if (e == std::string::npos) { err = "unterminated attribute"; return nullptr; }
            n->attrs.push_back({an, s.substr(i, e - i)});
            i = e + 1;
        }
        for (;;) {  // content
            size_t lt = s.find('<', i);
            if (lt == std::string::npos) { err = "unterminated element " + n->name; return nullptr; }
            n->text += s.substr(i, lt - i);
            i = lt;
            if (s.compare(i, 4, "<!--") == 0) {
                size_t e = s.find("-->", i + 4);
                if (e == std::string::npos) { err = "unterminated comment"; return nullptr; }
                i = e + 3;
                continue;
            }
            if (s.compare(i, 2, "</") == 0) {
                size_t e = s.find('>', i);
                if (e == std::string::npos) { err = "unterminated end tag"; return nullptr; }
                i = e + 1;
                return n;
            }
            auto k = element();
            if (!k) return nullptr;
            n->kids.push_back(std::move(k));
        }
    }
};

std::string dir_of(const std::string& path) {
    size_t p = path.find_last_of("/\\");
    return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}

bool read_file(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

// Wavefront OBJ: "v x y z" and "f a b c ..." (a, a/t, a/t/n, a//n; 1-based or
// negative), polygons split into fans.
bool read_obj(const std::string& path, std::vector<double>& X, std::vector<int>& F, std::string& err) {
    std::ifstream f(path);
    if (!f) { err = "cannot open " + path; return false; }
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string tag;
        ls >> tag;
        if (tag == "v") {
            double x, y, z;
            if (!(ls >> x >> y >> z)) { err = "bad vertex line in " + path; return false; }
            X.insert(X.end(), {x, y, z});
        } else if (tag == "f") {
            std::vector<int> poly;
            std::string tok;
            while (ls >> tok) {
                const int v = std::atoi(tok.c_str());
                const int nv = (int)X.size() / 3;
                const int id = v > 0 ? v - 1 : nv + v;
                if (v == 0 || id < 0 || id >= nv) { err = "bad face index in " + path; return false; }
                poly.push_back(id);
            }
            for (size_t k = 2; k < poly.size(); ++k) F.insert(F.end(), {poly[0], poly[k - 1], poly[k]});
        }
    }
    if (X.empty() || F.empty()) { err = "no vertices or faces in " + path; return false; }
    return true;
}

// tetgen .node / .ele; 0- or 1-based as the first record says
// (BaseTetMesh::readMeshFromTetFormat, Model/VolumetricMesh/BaseTetMesh.cpp:7-140)
bool read_tet(const std::string& node, const std::string& ele, std::vector<double>& X, std::vector<int>& T,
              std::string& err) {
    std::ifstream fn(node), fe(ele);
    if (!fn || !fe) { err = "cannot open " + node + " / " + ele; return false; }
    auto next = [](std::ifstream& f, std::string& line) {
        while (std::getline(f, line)) {
            size_t h = line.find('#');
            if (h != std::string::npos) line.resize(h);
            if (line.find_first_not_of(" \t\r") != std::string::npos) return true;
        }
        return false;
    };
    std::string line;
    if (!next(fn, line)) { err = "empty " + node; return false; }
    int np = 0, dim = 0;
    std::istringstream(line) >> np >> dim;
    if (np <= 0 || dim != 3) { err = "bad header in " + node; return false; }
    X.assign(3 * (size_t)np, 0.0);
    int base = -1;
    for (int k = 0; k < np; ++k) {
        if (!next(fn, line)) { err = "short " + node; return false; }
        std::istringstream ls(line);
        int id;
        double x, y, z;
        if (!(ls >> id >> x >> y >> z)) { err = "bad node line in " + node; return false; }
        if (base < 0) base = id == 0 ? 0 : 1;
        id -= base;
        if (id < 0 || id >= np) { err = "node index out of range in " + node; return false; }
        X[3 * (size_t)id] = x;
        X[3 * (size_t)id + 1] = y;
        X[3 * (size_t)id + 2] = z;
    }
    if (!next(fe, line)) { err = "empty " + ele; return false; }
    int nt = 0, per = 0;
    std::istringstream(line) >> nt >> per;
    if (nt <= 0 || per < 4) { err = "bad header in " + ele; return false; }
    T.assign(4 * (size_t)nt, 0);
    int ebase = -1;
    for (int k = 0; k < nt; ++k) {
        if (!next(fe, line)) { err = "short " + ele; return false; }
        std::istringstream ls(line);
        int id, v[4];
        if (!(ls >> id >> v[0] >> v[1] >> v[2] >> v[3])) { err = "bad element line in " + ele; return false; }
        if (ebase < 0) ebase = id == 0 ? 0 : 1;
        id -= ebase;
        if (id < 0 || id >= nt) { err = "element index out of range in " + ele; return false; }
        for (int q = 0; q < 4; ++q) {
            v[q] -= ebase;
            if (v[q] < 0 || v[q] >= np) { err = "element vertex out of range in " + ele; return false; }
            T[4 * (size_t)id + q] = v[q];
        }
    }
    return true;
}

void read_fixed(const std::string& path, std::vector<int>& pins) {
    std::ifstream f(path);
    if (!f) return;
    char ch = 0;
    int n = 0;
    f >> ch >> n;
    if (ch != 'c') return;
    for (int j = 0; j < n; ++j) {
        int v;
        if (!(f >> v)) break;
        pins.push_back(v);
    }
}

void box_centre(const std::vector<double>& X, double c[3], double ext[3]) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < X.size(); i += 3)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], X[i + k]);
            hi[k] = std::max(hi[k], X[i + k]);
        }
    for (int k = 0; k < 3; ++k) {
        c[k] = (lo[k] + hi[k]) / 2.0;
        ext[k] = hi[k] - lo[k];
    }
}

std::vector<double> numbers(const std::string& text) {
    std::istringstream ss(text);
    std::vector<double> v;
    double x;
    while (ss >> x) v.push_back(x);
    return v;
}

}  // namespace

struct pdipc_scene {
    struct Model {
        std::string name;
        int kind = 0;  // 0 cloth, 1 volumetric, 2 static
        std::vector<double> X;
        std::vector<int> F, T, pins;
        double density = 10.0, k[3] = {0, 0, 0};
        int patch_dim = 10;
    };
    std::vector<Model> models;
    bool has_dt = false, has_g = false, has_dhat = false, has_kappa = false;
    double dt = 0, g = 0, dhat = 0, kappa = 0;
};

extern "C" {

pdipc_status pdipc_scene_load(const char* config_path, pdipc_scene** out, char* err, int err_len) {
    auto fail = [&](pdipc_status st, const std::string& m) {
        if (err && err_len > 0) {
            std::strncpy(err, m.c_str(), (size_t)err_len - 1);
            err[err_len - 1] = 0;
        }
        return st;
    };
    if (!config_path || !out) return fail(PDIPC_ERR_ARG, "null argument");
    *out = nullptr;
    try {
        std::string text;
        if (!read_file(config_path, text)) return fail(PDIPC_ERR_IO, std::string("cannot read ") + config_path);
        XParser xp(text);
        std::unique_ptr<XNode> root = xp.element();
        if (!root) return fail(PDIPC_ERR_IO, "config: " + xp.err);
        const XNode* sim = root->name == "simulator" ? root.get() : root->child("simulator");
        if (!sim) return fail(PDIPC_ERR_IO, "config has no <simulator> element");
        const std::string dir = dir_of(config_path);
        auto sc = std::make_unique<pdipc_scene>();
        for (auto& kid : sim->kids) {
            const XNode& e = *kid;
            const std::vector<double> v = numbers(e.text);
            if (e.name == "timeStep" && !v.empty()) { sc->has_dt = true; sc->dt = v[0]; }
            else if (e.name == "gravity" && !v.empty()) { sc->has_g = true; sc->g = v[0]; }
            else if (e.name == "dhat" && !v.empty()) { sc->has_dhat = true; sc->dhat = v[0]; }
            else if (e.name == "kappa" && !v.empty()) { sc->has_kappa = true; sc->kappa = v[0]; }
            else if (e.name == "object" || e.name == "static_object") {
                if (e.attrs.empty() || e.attrs[0].first != "name")
                    return fail(PDIPC_ERR_IO, "<" + e.name + "> must start with a name attribute");
                pdipc_scene::Model m;
                m.name = e.attrs[0].second;
                bool tet = false, uniform = true, origin = true;
                auto off = [](const std::string& s) { return s == "off" || s == "false" || s == "0"; };
                for (auto& a : e.attrs) {
                    if (a.first == "volumetric_mesh" && a.second == "tet") tet = true;
                    if (a.first == "uniform") uniform = !off(a.second);
                    if (a.first == "origin") origin = !off(a.second);
                }
                int type = 1;
                double scale[3] = {1, 1, 1}, trans[3] = {0, 0, 0}, rot[3] = {0, 0, 0};
                for (auto& c : e.kids) {
                    const std::vector<double> n = numbers(c->text);
                    if (c->name == "type" && n.size() >= 4) {
                        type = (int)n[0];
                        m.k[0] = n[1];
                        m.k[1] = n[2];
                        m.k[2] = n[3];
                    } else if (c->name == "patchDim" && !n.empty()) m.patch_dim = (int)n[0];
                    else if (c->name == "scale" && n.size() >= 3) std::copy(n.begin(), n.begin() + 3, scale);
                    else if (c->name == "translation" && n.size() >= 3) std::copy(n.begin(), n.begin() + 3, trans);
                    else if (c->name == "rotation" && n.size() >= 3) std::copy(n.begin(), n.begin() + 3, rot);
                    else if (c->name == "density" && !n.empty()) m.density = n[0];
                }
                const std::string base = dir + m.name + "/" + m.name;
                std::string rerr;
                if (!read_obj(base + ".obj", m.X, m.F, rerr)) return fail(PDIPC_ERR_IO, rerr);
                std::vector<double> TX;  // tet points move with the surface
                if (tet && !read_tet(base + ".node", base + ".ele", TX, m.T, rerr)) return fail(PDIPC_ERR_IO, rerr);
                auto apply = [&](auto&& f) {
                    for (size_t q = 0; q < m.X.size(); q += 3) f(&m.X[q]);
                    for (size_t q = 0; q < TX.size(); q += 3) f(&TX[q]);
                };
                double c[3], ext[3];
                if (origin) {
                    box_centre(m.X, c, ext);
                    apply([&](double* p) { for (int k = 0; k < 3; ++k) p[k] -= c[k]; });
                }
                if (uniform) {
                    box_centre(m.X, c, ext);
                    double div = std::max(ext[0], std::max(ext[1], ext[2]));
                    if (std::fabs(div) < 1e-6) div = 1.0;
                    apply([&](double* p) { for (int k = 0; k < 3; ++k) p[k] /= div; });
                }
                box_centre(m.X, c, ext);
                apply([&](double* p) { for (int k = 0; k < 3; ++k) p[k] = (p[k] - c[k]) * scale[k] + c[k]; });
                apply([&](double* p) { for (int k = 0; k < 3; ++k) p[k] += trans[k]; });
                if (rot[0] != 0.0 || rot[1] != 0.0 || rot[2] != 0.0) {
                    const double d2r = 3.14159265358979323846 / 180.0;
                    const double cx = std::cos(rot[0] * d2r), sx = std::sin(rot[0] * d2r);
                    const double cy = std::cos(rot[1] * d2r), sy = std::sin(rot[1] * d2r);
                    const double cz = std::cos(rot[2] * d2r), sz = std::sin(rot[2] * d2r);
                    const double R[3][3] = {{cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx},
                                            {sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx},
                                            {-sy, cy * sx, cy * cx}};
                    box_centre(m.X, c, ext);
                    apply([&](double* p) {
                        const double d[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
                        for (int k = 0; k < 3; ++k) p[k] = c[k] + R[k][0] * d[0] + R[k][1] * d[1] + R[k][2] * d[2];
                    });
                }
                if (e.name == "static_object") m.kind = 2;
                else if (type == 1) {
                    if (!tet) return fail(PDIPC_ERR_IO, m.name + ": <type> 1 needs volumetric_mesh=\"tet\"");
                    m.kind = 1;
                } else {
                    m.kind = 0;
                }
                if (m.kind == 1) m.X.swap(TX);  // a volumetric model simulates its tet points
                else m.T.clear();
                if (m.kind != 2) read_fixed(dir + m.name + "/fixed_points.txt", m.pins);
                sc->models.push_back(std::move(m));
            }
        }
        *out = sc.release();
        return PDIPC_OK;
    } catch (const std::bad_alloc&) {
        return fail(PDIPC_ERR_ALLOC, "host allocation failed");
    }
}

int pdipc_scene_model_count(const pdipc_scene* s) { return s ? (int)s->models.size() : 0; }

pdipc_status pdipc_scene_get_model(const pdipc_scene* s, int i, pdipc_scene_model* out) {
    if (!s || !out || i < 0 || i >= (int)s->models.size()) return PDIPC_ERR_ARG;
    const pdipc_scene::Model& m = s->models[i];
    out->name = m.name.c_str();
    out->kind = m.kind;
    out->nv = (int)m.X.size() / 3;
    out->nf = (int)m.F.size() / 3;
    out->nt = (int)m.T.size() / 4;
    out->npins = (int)m.pins.size();
    out->X = m.X.data();
    out->F = m.F.data();
    out->T = m.T.empty() ? nullptr : m.T.data();
    out->pins = m.pins.empty() ? nullptr : m.pins.data();
    out->density = m.density;
    out->k[0] = m.k[0];
    out->k[1] = m.k[1];
    out->k[2] = m.k[2];
    out->patch_dim = m.patch_dim;
    return PDIPC_OK;
}

pdipc_status pdipc_scene_apply_params(const pdipc_scene* s, pdipc_params* p) {
    if (!s || !p) return PDIPC_ERR_ARG;
    if (s->has_dt) p->time_step = s->dt;
    if (s->has_g) p->gravity = s->g;
    if (s->has_dhat) p->dhat = s->dhat;
    if (s->has_kappa) p->kappa = s->kappa;
    return PDIPC_OK;
}

pdipc_status pdipc_scene_add_models(const pdipc_scene* s, pdipc_ctx* ctx) {
    if (!s || !ctx) return PDIPC_ERR_ARG;
    for (const auto& m : s->models) {
        const int nv = (int)m.X.size() / 3;
        const int* pins = m.pins.empty() ? nullptr : m.pins.data();
        pdipc_status st;
        if (m.kind == 2) st = pdipc_add_static(ctx, m.X.data(), nv, m.F.data(), (int)m.F.size() / 3, m.patch_dim);
        else if (m.kind == 1)
            st = pdipc_add_volumetric(ctx, m.X.data(), nv, m.T.data(), (int)m.T.size() / 4, m.density, m.k[0], m.k[1],
                                      pins, (int)m.pins.size(), m.k[2], m.patch_dim);
        else
            st = pdipc_add_cloth(ctx, m.X.data(), nv, m.F.data(), (int)m.F.size() / 3, m.density, m.k[0], m.k[1],
                                 pins, (int)m.pins.size(), m.k[2], m.patch_dim);
        if (st != PDIPC_OK) return st;
    }
    return PDIPC_OK;
}

void pdipc_scene_free(pdipc_scene* s) { delete s; }

}  // extern "C"
