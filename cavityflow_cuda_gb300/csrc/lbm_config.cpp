// lbm_config.cpp -- reads the reference's XML configuration file
// (configurations/*.xml; the schema of src/CConfiguration.cpp:54-160) into
// lbm_configuration, with a small XML reader written for that schema:
// nested elements with text content, comments, the XML declaration and
// attributes (ignored).  Numbers are converted with atof/atoi as the
// reference does, and the reference's parameter checks
// (src/CConfiguration.cpp:174-197, asserts there) return LBM_ERR_CONFIG.
// As in the reference built without MPI, subdomain-num is not read and the
// domain is one subdomain (subdomain_num = 1, 1, 1).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <limits>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_internal.h"

using lbm_detail::fail;

namespace {

struct Node {
    std::string name;
    std::string text;
    std::vector<std::unique_ptr<Node>> children;

    const Node* child(const char* n) const
    {
        for (const auto& c : children)
            if (c->name == n) return c.get();
        return nullptr;
    }
};

class Parser {
public:
    explicit Parser(const std::string& s) : s_(s) {}

    bool parse(Node& root, std::string& err)
    {
        skip_misc();
        if (!element(root, err, 0)) return false;
        skip_misc();
        if (i_ != s_.size()) {
            err = "trailing content after the root element";
            return false;
        }
        return true;
    }

private:
    const std::string& s_;
    size_t i_ = 0;

    bool starts(const char* t) const { return s_.compare(i_, std::strlen(t), t) == 0; }

    void skip_ws()
    {
        while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
    }

    // whitespace, comments, processing instructions (<?xml ...?>) and <!DOCTYPE>
    void skip_misc()
    {
        for (;;) {
            skip_ws();
            if (starts("<!--")) {
                const size_t e = s_.find("-->", i_ + 4);
                i_ = e == std::string::npos ? s_.size() : e + 3;
            } else if (starts("<?")) {
                const size_t e = s_.find("?>", i_ + 2);
                i_ = e == std::string::npos ? s_.size() : e + 2;
            } else if (starts("<!")) {
                const size_t e = s_.find('>', i_ + 2);
                i_ = e == std::string::npos ? s_.size() : e + 1;
            } else {
                return;
            }
        }
    }

    // The schema nests four levels deep; deeper documents are refused rather
    // than recursed into without bound.
    static constexpr int kMaxDepth = 64;

    bool element(Node& n, std::string& err, int depth)
    {
        if (depth > kMaxDepth) {
            err = "elements nested deeper than 64 levels";
            return false;
        }
        if (i_ >= s_.size() || s_[i_] != '<') {
            err = "expected an element";
            return false;
        }
        ++i_;
        const size_t b = i_;
        while (i_ < s_.size() && !std::isspace((unsigned char)s_[i_]) && s_[i_] != '>' && s_[i_] != '/') ++i_;
        n.name = s_.substr(b, i_ - b);
        if (n.name.empty()) {
            err = "empty element name";
            return false;
        }
        // attributes are not used by the schema: skip to the end of the tag
        while (i_ < s_.size() && s_[i_] != '>' && !(s_[i_] == '/' && i_ + 1 < s_.size() && s_[i_ + 1] == '>')) {
            if (s_[i_] == '"' || s_[i_] == '\'') {
                const char q = s_[i_];
                const size_t e = s_.find(q, i_ + 1);
                i_ = e == std::string::npos ? s_.size() : e + 1;
            } else {
                ++i_;
            }
        }
        if (i_ >= s_.size()) {
            err = "unterminated tag <" + n.name + ">";
            return false;
        }
        if (s_[i_] == '/') {  // <name/>
            i_ += 2;
            return true;
        }
        ++i_;
        for (;;) {
            if (i_ >= s_.size()) {
                err = "missing </" + n.name + ">";
                return false;
            }
            if (starts("<!--") || starts("<?")) {
                skip_misc();
                continue;
            }
            if (starts("</")) {
                i_ += 2;
                const size_t b2 = i_;
                while (i_ < s_.size() && s_[i_] != '>') ++i_;
                if (i_ >= s_.size()) {
                    err = "unterminated </" + n.name + ">";
                    return false;
                }
                std::string close = s_.substr(b2, i_ - b2);
                while (!close.empty() && std::isspace((unsigned char)close.back())) close.pop_back();
                if (close != n.name) {
                    err = "</" + close + "> closes <" + n.name + ">";
                    return false;
                }
                ++i_;
                return true;
            }
            if (s_[i_] == '<') {
                auto c = std::make_unique<Node>();
                if (!element(*c, err, depth + 1)) return false;
                n.children.push_back(std::move(c));
            } else {
                const size_t e = s_.find('<', i_);
                n.text += s_.substr(i_, (e == std::string::npos ? s_.size() : e) - i_);
                i_ = e == std::string::npos ? s_.size() : e;
            }
        }
    }
};

std::string trim(const std::string& t)
{
    size_t a = 0, b = t.size();
    while (a < b && std::isspace((unsigned char)t[a])) ++a;
    while (b > a && std::isspace((unsigned char)t[b - 1])) --b;
    return t.substr(a, b - a);
}

// Follows a path of child names; the reference dereferences each step, so a
// missing element is a configuration error here.
const Node* at(const Node* n, std::initializer_list<const char*> path, std::string& missing)
{
    std::string where = n->name;
    for (const char* p : path) {
        where += "/";
        where += p;
        n = n ? n->child(p) : nullptr;
        if (!n) {
            if (missing.empty()) missing = where;
            return nullptr;
        }
    }
    return n;
}

double num(const Node* root, std::initializer_list<const char*> path, std::string& missing)
{
    const Node* n = at(root, path, missing);
    return n ? std::atof(trim(n->text).c_str()) : 0.0;
}

int inum(const Node* root, std::initializer_list<const char*> path, std::string& missing)
{
    const Node* n = at(root, path, missing);
    return n ? std::atoi(trim(n->text).c_str()) : 0;
}

void str(const Node* root, std::initializer_list<const char*> path, std::string& missing, char* out, size_t cap)
{
    const Node* n = at(root, path, missing);
    const std::string v = n ? trim(n->text) : std::string();
    std::snprintf(out, cap, "%s", v.c_str());
}

}  // namespace

namespace {

int read_configuration(const char* path, lbm_configuration* c)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(LBM_ERR_IO, "cannot open configuration \"%s\"", path);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    Node root;
    std::string err;
    if (!Parser(text).parse(root, err)) return fail(LBM_ERR_CONFIG, "%s: XML error: %s", path, err.c_str());
    if (root.name != "lbm-configuration")
        return fail(LBM_ERR_CONFIG, "%s: root element is <%s>, not <lbm-configuration>", path, root.name.c_str());
    std::memset(c, 0, sizeof(*c));
    std::string missing;
    const Node* r = &root;
    const char* xyz[3] = {"x", "y", "z"};
    for (int d = 0; d < 3; ++d) {
        c->velocity[d] = num(r, {"physics", "velocity", xyz[d]}, missing);
        c->acceleration[d] = num(r, {"physics", "acceleration", xyz[d]}, missing);
        c->domain_size[d] = inum(r, {"grid", "domain-size", xyz[d]}, missing);
        c->domain_length[d] = num(r, {"grid", "domian-length", xyz[d]}, missing);  // sic, the schema's spelling
        c->subdomain_num[d] = 1;  // not read without MPI (src/CConfiguration.cpp:86-92)
        c->cpu_alpha_block[d] = inum(r, {"cpu", "block-configuration", "alpha-block-configuration", xyz[d]}, missing);
        c->cpu_beta_block[d] = inum(r, {"cpu", "block-configuration", "beta-block-configuration", xyz[d]}, missing);
        c->gpu_init_block[d] = inum(r, {"gpu", "grid-configuration", "init-grid-configuration", xyz[d]}, missing);
        c->gpu_alpha_block[d] = inum(r, {"gpu", "grid-configuration", "alpha-grid-configuration", xyz[d]}, missing);
        c->gpu_beta_block[d] = inum(r, {"gpu", "grid-configuration", "beta-grid-configuration", xyz[d]}, missing);
    }
    c->viscosity = num(r, {"physics", "viscosity"}, missing);
    c->max_velocity = num(r, {"physics", "max-velocity"}, missing);
    c->max_acceleration = num(r, {"physics", "max-acceleration"}, missing);
    c->cpu_subdomain_ratio = num(r, {"grid", "cpu-subdomain-ratio"}, missing);
    c->loops = inum(r, {"simulation", "loops"}, missing);
    c->timestep = num(r, {"simulation", "timestep"}, missing);
    c->do_benchmark = inum(r, {"simulation", "benchmark", "do"}, missing);
    c->do_logging = inum(r, {"simulation", "logging", "do"}, missing);
    c->do_validation = inum(r, {"simulation", "validation", "do"}, missing);
    c->do_visualization = inum(r, {"simulation", "visualization", "do"}, missing);
    c->visualization_rate = inum(r, {"simulation", "visualization", "rate"}, missing);
    str(r, {"simulation", "benchmark", "output-dir"}, missing, c->benchmark_dir, sizeof(c->benchmark_dir));
    str(r, {"simulation", "logging", "output-dir"}, missing, c->logging_dir, sizeof(c->logging_dir));
    str(r, {"simulation", "validation", "output-dir"}, missing, c->validation_dir, sizeof(c->validation_dir));
    str(r, {"simulation", "visualization", "output-dir"}, missing, c->visualization_dir, sizeof(c->visualization_dir));
    if (!missing.empty()) return fail(LBM_ERR_CONFIG, "%s: element <%s> is missing", path, missing.c_str());

    // src/CConfiguration.cpp:174-197
    const char* bad = nullptr;
    for (int d = 0; d < 3 && !bad; ++d) {
        if (c->domain_size[d] <= 0) bad = "domain-size must be positive";
        else if (!(c->domain_length[d] > 0)) bad = "domian-length must be positive";
        else if (c->cpu_alpha_block[d] <= 0 || c->cpu_beta_block[d] <= 0) bad = "cpu block configuration must be positive";
        else if (c->gpu_init_block[d] <= 0 || c->gpu_alpha_block[d] <= 0 || c->gpu_beta_block[d] <= 0)
            bad = "gpu grid configuration must be positive";
    }
    if (!bad && !(c->timestep > 0)) bad = "timestep must be positive";
    if (!bad && !(c->max_velocity > 0)) bad = "max-velocity must be positive";
    if (!bad && !(c->max_acceleration > 0)) bad = "max-acceleration must be positive";
    if (!bad && !(c->cpu_subdomain_ratio >= 0 && c->cpu_subdomain_ratio <= 1)) bad = "cpu-subdomain-ratio not in [0,1]";
    if (!bad && c->visualization_rate <= 0) bad = "visualization rate must be positive";
    if (!bad) {
        // Equal cell lengths on all axes.  The reference compares in its own
        // precision against that precision's epsilon; the reader does not know
        // the precision, so a configuration must pass both comparisons.
        const float lx = (float)c->domain_length[0] / (float)c->domain_size[0];
        const float ly = (float)c->domain_length[1] / (float)c->domain_size[1];
        const float lz = (float)c->domain_length[2] / (float)c->domain_size[2];
        const float fe = std::numeric_limits<float>::epsilon();
        const double dx = c->domain_length[0] / c->domain_size[0];
        const double dy = c->domain_length[1] / c->domain_size[1];
        const double dz = c->domain_length[2] / c->domain_size[2];
        const double de = std::numeric_limits<double>::epsilon();
        if (std::fabs(lx - ly) >= fe || std::fabs(ly - lz) >= fe || std::fabs(lz - lx) >= fe ||
            std::fabs(dx - dy) >= de || std::fabs(dy - dz) >= de || std::fabs(dz - dx) >= de)
            bad = "cells must be cubes (domian-length / domain-size equal on every axis)";
    }
    for (int k = 0; k < 3 && !bad; ++k) {
        const int32_t* g = k == 0 ? c->gpu_init_block : k == 1 ? c->gpu_alpha_block : c->gpu_beta_block;
        if ((long long)g[0] * g[1] * g[2] > 1024) bad = "gpu grid configuration above 1024 threads";
    }
    if (bad) return fail(LBM_ERR_CONFIG, "%s: %s", path, bad);
    return LBM_OK;
}

}  // namespace

extern "C" int lbm_read_configuration(const char* path, lbm_configuration* c)
{
    if (!path || !c) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    try {  // no C++ exception may cross the C interface (a file too large for memory, say)
        return read_configuration(path, c);
    } catch (const std::exception& e) {
        return fail(LBM_ERR_CONFIG, "%s: %s", path, e.what());
    }
}

extern "C" int lbm_configuration_physical(const lbm_configuration* c, lbm_physical* out)
{
    if (!c || !out) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    for (int d = 0; d < 3; ++d) {
        out->velocity[d] = c->velocity[d];
        out->acceleration[d] = c->acceleration[d];
        // one domain on one GPU, as the reference built without MPI sets
        // numOfSubdomains to 1 (src/CConfiguration.cpp:86-92, src/CManager.cpp:27-58)
        out->domain_size[d] = c->domain_size[d];
        out->domain_length[d] = c->domain_length[d];
    }
    out->viscosity = c->viscosity;
    out->max_velocity = c->max_velocity;
    out->max_acceleration = c->max_acceleration;
    out->timestep = c->timestep;
    return LBM_OK;
}
