// Host object model and XML serialization of the ATM path.
#include "model.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>

namespace atm {

const char* const kVersion = "0.3.1";

static const char* const kGlobalNames[NUM_GLOBALS] = {"ATMLambda1", "ATMLambda2", "ATMAlpha",
                                                     "ATMU0",      "ATMW0",      "ATMUmax",
                                                     "ATMUbcore",  "ATMAcore",   "ATMDirection"};

const char* global_name(int which) {
    if (which < 0 || which >= NUM_GLOBALS) return nullptr;
    return kGlobalNames[which];
}

int global_index(const std::string& name) {
    for (int k = 0; k < NUM_GLOBALS; k++)
        if (name == kGlobalNames[k]) return k;
    return -1;
}

ATMMetaForce::ATMMetaForce(double lambda1, double lambda2, double alpha, double u0, double w0, double umax,
                           double ubcore, double acore, double direction, const std::vector<int>& g)
    : groups(g) {
    double d[NUM_GLOBALS] = {lambda1, lambda2, alpha, u0, w0, umax, ubcore, acore, direction};
    for (int k = 0; k < NUM_GLOBALS; k++) defaults[k] = d[k];
}

int ATMMetaForce::addParticle(int particle, double dx, double dy, double dz) {
    // ATMMetaForce.cpp:12-15
    particles.push_back(ParticleInfo{particle, dx, dy, dz});
    return (int)particles.size() - 1;
}

void ATMMetaForce::getParticleParameters(int index, int& particle, double& dx, double& dy, double& dz) const {
    // ATMMetaForce.cpp:17-24 (ASSERT_VALID_INDEX)
    if (index < 0 || index >= (int)particles.size()) throw Error(2, "Index out of range");
    const ParticleInfo& p = particles[index];
    particle = p.particle;
    dx = p.dx;
    dy = p.dy;
    dz = p.dz;
}

void ATMMetaForce::setParticleParameters(int index, int particle, double dx, double dy, double dz) {
    // ATMMetaForce.cpp:26-32
    if (index < 0 || index >= (int)particles.size()) throw Error(2, "Index out of range");
    particles[index] = ParticleInfo{particle, dx, dy, dz};
}

void ATMMetaForce::setForceGroup(int g) {
    // OpenMM Force::setForceGroup accepts 0..31
    if (g < 0 || g > 31) throw Error(1, "Force group must be between 0 and 31");
    forceGroup = g;
}

int NonbondedForce::addParticle(double q, double sig, double eps) {
    charge.push_back(q);
    sigma.push_back(sig);
    epsilon.push_back(eps);
    return (int)charge.size() - 1;
}

int NonbondedForce::addException(int i, int j, double qq, double sig, double eps) {
    if (i == j) throw Error(1, "An exception must involve two different particles");
    exceptions.push_back(Exception{i, j, qq, sig, eps});
    return (int)exceptions.size() - 1;
}

void pme_parameters(double cutoff, double tol, const double* box, double& alpha, int* grid) {
    alpha = std::sqrt(-std::log(2.0 * tol)) / cutoff;
    for (int a = 0; a < 3; a++) {
        int g = (int)std::ceil(2.0 * alpha * box[a] / (3.0 * std::pow(tol, 0.2)));
        grid[a] = g < 6 ? 6 : g;
    }
}

// ---------------------------------------------------------------------------
// XML.  Attribute set and child layout follow ATMMetaForceProxy.cpp:11-40;
// doubles are written with 17 significant digits so that a round trip is exact
// (TestSerializeATMMetaForce.cpp:49-75 compares with ASSERT_EQUAL).
// ---------------------------------------------------------------------------

static std::string fmt_double(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}

static std::string xml_escape(const std::string& s) {
    std::string o;
    for (char c : s) {
        switch (c) {
            case '&': o += "&amp;"; break;
            case '<': o += "&lt;"; break;
            case '>': o += "&gt;"; break;
            case '"': o += "&quot;"; break;
            case '\'': o += "&apos;"; break;
            default: o += c;
        }
    }
    return o;
}

std::string serialize(const ATMMetaForce& f) {
    std::ostringstream o;
    o << "<?xml version=\"1.0\" ?>\n";
    o << "<Force aCore=\"" << fmt_double(f.defaults[ACORE]) << "\" alpha=\"" << fmt_double(f.defaults[ALPHA])
      << "\" direction=\"" << fmt_double(f.defaults[DIRECTION]) << "\" forceGroup=\"" << f.forceGroup
      << "\" lambda1=\"" << fmt_double(f.defaults[LAMBDA1]) << "\" lambda2=\"" << fmt_double(f.defaults[LAMBDA2])
      << "\" name=\"" << xml_escape(f.name) << "\" type=\"ATMMetaForce\" u0=\"" << fmt_double(f.defaults[U0])
      << "\" uMax=\"" << fmt_double(f.defaults[UMAX]) << "\" ubCore=\"" << fmt_double(f.defaults[UBCORE])
      << "\" version=\"0\" w0=\"" << fmt_double(f.defaults[W0]) << "\">\n";
    o << "\t<VariableForceGroups>\n";
    for (int g : f.groups) o << "\t\t<Parameter group=\"" << g << "\"/>\n";
    o << "\t</VariableForceGroups>\n";
    o << "\t<Particles>\n";
    for (const auto& p : f.particles)
        o << "\t\t<Particle dx=\"" << fmt_double(p.dx) << "\" dy=\"" << fmt_double(p.dy) << "\" dz=\""
          << fmt_double(p.dz) << "\" particle=\"" << p.particle << "\"/>\n";
    o << "\t</Particles>\n";
    o << "</Force>\n";
    return o.str();
}

// Minimal XML element reader: enough for OpenMM's serializer output
// (elements, attributes, self-closing tags, declarations, comments).
namespace {
struct Node {
    std::string tag;
    std::map<std::string, std::string> attr;
    std::vector<Node> kids;
};

struct Parser {
    const std::string& s;
    size_t p = 0;
    explicit Parser(const std::string& str) : s(str) {}
    [[noreturn]] void fail(const char* what) { throw Error(7, std::string("XML parse error: ") + what); }
    void ws() {
        while (p < s.size() && std::isspace((unsigned char)s[p])) p++;
    }
    void skip_misc() {
        for (;;) {
            ws();
            if (s.compare(p, 4, "<!--") == 0) {
                size_t e = s.find("-->", p);
                if (e == std::string::npos) fail("unterminated comment");
                p = e + 3;
            } else if (s.compare(p, 2, "<?") == 0) {
                size_t e = s.find("?>", p);
                if (e == std::string::npos) fail("unterminated declaration");
                p = e + 2;
            } else {
                break;
            }
        }
    }
    static std::string unescape(const std::string& v) {
        std::string o;
        for (size_t k = 0; k < v.size(); k++) {
            if (v[k] != '&') {
                o += v[k];
                continue;
            }
            size_t e = v.find(';', k);
            std::string ent = v.substr(k + 1, e - k - 1);
            if (ent == "amp") o += '&';
            else if (ent == "lt") o += '<';
            else if (ent == "gt") o += '>';
            else if (ent == "quot") o += '"';
            else if (ent == "apos") o += '\'';
            else o += "&" + ent + ";";
            k = e;
        }
        return o;
    }
    Node element() {
        skip_misc();
        if (p >= s.size() || s[p] != '<') fail("expected element");
        p++;
        Node n;
        while (p < s.size() && !std::isspace((unsigned char)s[p]) && s[p] != '>' && s[p] != '/') n.tag += s[p++];
        for (;;) {
            ws();
            if (p >= s.size()) fail("unterminated tag");
            if (s[p] == '/') {
                if (s.compare(p, 2, "/>") != 0) fail("bad tag end");
                p += 2;
                return n;
            }
            if (s[p] == '>') {
                p++;
                break;
            }
            std::string key;
            while (p < s.size() && s[p] != '=' && !std::isspace((unsigned char)s[p])) key += s[p++];
            ws();
            if (p >= s.size() || s[p] != '=') fail("expected '='");
            p++;
            ws();
            if (p >= s.size() || (s[p] != '"' && s[p] != '\'')) fail("expected quote");
            char q = s[p++];
            size_t e = s.find(q, p);
            if (e == std::string::npos) fail("unterminated attribute");
            n.attr[key] = unescape(s.substr(p, e - p));
            p = e + 1;
        }
        for (;;) {
            skip_misc();
            if (s.compare(p, 2, "</") == 0) {
                size_t e = s.find('>', p);
                if (e == std::string::npos) fail("unterminated end tag");
                p = e + 1;
                return n;
            }
            if (p >= s.size()) fail("unexpected end of document");
            if (s[p] == '<') {
                n.kids.push_back(element());
            } else {
                while (p < s.size() && s[p] != '<') p++;  // text content is ignored
            }
        }
    }
};

const std::string& req(const Node& n, const char* key) {
    auto it = n.attr.find(key);
    if (it == n.attr.end()) throw Error(7, std::string("Missing attribute: ") + key);
    return it->second;
}

double to_double(const std::string& v) {
    char* end = nullptr;
    double d = std::strtod(v.c_str(), &end);
    if (end == v.c_str()) throw Error(7, "Bad number: " + v);
    return d;
}

int to_int(const std::string& v) {
    char* end = nullptr;
    long d = std::strtol(v.c_str(), &end, 10);
    if (end == v.c_str()) throw Error(7, "Bad integer: " + v);
    return (int)d;
}

const Node& child(const Node& n, const char* tag) {
    for (const auto& k : n.kids)
        if (k.tag == tag) return k;
    throw Error(7, std::string("Missing element: ") + tag);
}
}  // namespace

std::unique_ptr<ATMMetaForce> deserialize(const std::string& xml) {
    Parser P(xml);
    Node root = P.element();
    // ATMMetaForceProxy.cpp:43-44: only version 0 is understood
    if (to_int(req(root, "version")) != 0) throw Error(7, "Unsupported version");
    auto ti = root.attr.find("type");
    if (ti != root.attr.end() && ti->second != "ATMMetaForce") throw Error(7, "Not an ATMMetaForce: " + ti->second);
    std::vector<int> groups;
    for (const auto& g : child(root, "VariableForceGroups").kids) groups.push_back(to_int(req(g, "group")));
    std::unique_ptr<ATMMetaForce> f(new ATMMetaForce(
        to_double(req(root, "lambda1")), to_double(req(root, "lambda2")), to_double(req(root, "alpha")),
        to_double(req(root, "u0")), to_double(req(root, "w0")), to_double(req(root, "uMax")),
        to_double(req(root, "ubCore")), to_double(req(root, "aCore")), to_double(req(root, "direction")), groups));
    auto fg = root.attr.find("forceGroup");
    f->setForceGroup(fg == root.attr.end() ? 0 : to_int(fg->second));
    auto nm = root.attr.find("name");
    if (nm != root.attr.end()) f->setName(nm->second);
    for (const auto& p : child(root, "Particles").kids)
        f->addParticle(to_int(req(p, "particle")), to_double(req(p, "dx")), to_double(req(p, "dy")),
                       to_double(req(p, "dz")));
    return f;
}

}  // namespace atm
