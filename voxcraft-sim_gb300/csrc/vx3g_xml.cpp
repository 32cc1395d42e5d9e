// vx3g_xml.cpp -- small XML reader for VXA/VXD documents (see vx3g_xml.h).
#include "vx3g_xml.h"

#include <cctype>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace vx3g {
namespace xml {

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

std::unique_ptr<Node> Node::clone() const {
    auto n = std::make_unique<Node>();
    n->name = name;
    n->attrs = attrs;
    n->text = text;
    for (auto &c : children) n->children.push_back(c->clone());
    return n;
}

namespace {

struct Parser {
    const std::string &s;
    size_t i = 0;
    explicit Parser(const std::string &src) : s(src) {}

    [[noreturn]] void error(const char *what) {
        throw std::runtime_error(std::string("XML parse error: ") + what + " at offset " + std::to_string(i));
    }
    bool starts(const char *p) const { return s.compare(i, std::strlen(p), p) == 0; }
    void skip_ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    void skip_until(const char *end) {
        size_t j = s.find(end, i);
        if (j == std::string::npos) error("unterminated construct");
        i = j + std::strlen(end);
    }
    std::string name() {
        size_t a = i;
        while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == '.' ||
                                s[i] == ':'))
            i++;
        if (a == i) error("expected a name");
        return s.substr(a, i - a);
    }
    static std::string unescape(const std::string &t) {
        std::string o;
        for (size_t k = 0; k < t.size(); k++) {
            if (t[k] != '&') {
                o += t[k];
                continue;
            }
            size_t e = t.find(';', k);
            if (e == std::string::npos) {
                o += t[k];
                continue;
            }
            std::string ent = t.substr(k + 1, e - k - 1);
            if (ent == "lt") o += '<';
            else if (ent == "gt") o += '>';
            else if (ent == "amp") o += '&';
            else if (ent == "quot") o += '"';
            else if (ent == "apos") o += '\'';
            else if (!ent.empty() && ent[0] == '#') o += (char)std::strtol(ent.c_str() + (ent[1] == 'x' ? 2 : 1), nullptr, ent[1] == 'x' ? 16 : 10);
            else o += "&" + ent + ";";
            k = e;
        }
        return o;
    }
    void misc() {  // comments, processing instructions, doctype
        for (;;) {
            skip_ws();
            if (starts("<?")) skip_until("?>");
            else if (starts("<!--")) skip_until("-->");
            else if (starts("<!DOCTYPE")) skip_until(">");
            else break;
        }
    }
    std::unique_ptr<Node> element() {
        if (!starts("<")) error("expected '<'");
        i++;
        auto n = std::make_unique<Node>();
        n->name = name();
        for (;;) {
            skip_ws();
            if (starts("/>")) {
                i += 2;
                return n;
            }
            if (starts(">")) {
                i++;
                break;
            }
            std::string an = name();
            skip_ws();
            if (i >= s.size() || s[i] != '=') error("expected '='");
            i++;
            skip_ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) error("expected quote");
            char q = s[i++];
            size_t e = s.find(q, i);
            if (e == std::string::npos) error("unterminated attribute");
            n->attrs.emplace_back(an, unescape(s.substr(i, e - i)));
            i = e + 1;
        }
        for (;;) {
            if (i >= s.size()) error("unterminated element");
            if (starts("</")) {
                i += 2;
                std::string en = name();
                if (en != n->name) error("mismatched end tag");
                skip_ws();
                if (!starts(">")) error("expected '>'");
                i++;
                return n;
            }
            if (starts("<![CDATA[")) {
                i += 9;
                size_t e = s.find("]]>", i);
                if (e == std::string::npos) error("unterminated CDATA");
                n->text += s.substr(i, e - i);
                i = e + 3;
            } else if (starts("<!--")) {
                skip_until("-->");
            } else if (starts("<?")) {
                skip_until("?>");
            } else if (starts("<")) {
                n->children.push_back(element());
            } else {
                size_t e = s.find('<', i);
                if (e == std::string::npos) e = s.size();
                n->text += unescape(s.substr(i, e - i));
                i = e;
            }
        }
    }
};

std::vector<std::string> split_path(const std::string &p) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : p) {
        if (c == '.') {
            out.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    out.push_back(cur);
    return out;
}

}  // namespace

std::unique_ptr<Node> parse(const std::string &text) {
    Parser p(text);
    auto root = std::make_unique<Node>();
    root->name = "";
    p.misc();
    while (p.i < text.size()) {
        root->children.push_back(p.element());
        p.misc();
    }
    return root;
}

std::unique_ptr<Node> parse_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return parse(ss.str());
}

const Node *find(const Node *root, const std::string &path) {
    const Node *n = root;
    for (auto &k : split_path(path)) {
        if (!n) return nullptr;
        n = n->child(k);
    }
    return n;
}

Node *find_or_create(Node *root, const std::string &path) {
    Node *n = root;
    for (auto &k : split_path(path)) {
        Node *c = n->child(k);
        if (!c) {
            n->children.push_back(std::make_unique<Node>());
            c = n->children.back().get();
            c->name = k;
        }
        n = c;
    }
    return n;
}

bool get_double(const Node *root, const std::string &path, double *out) {
    const Node *n = find(root, path);
    if (!n) return false;
    std::string t = trim(n->text);
    if (t.empty()) return false;
    char *end = nullptr;
    double v = std::strtod(t.c_str(), &end);
    if (end == t.c_str()) return false;
    *out = v;
    return true;
}

double get_double(const Node *root, const std::string &path, double dflt) {
    double v;
    return get_double(root, path, &v) ? v : dflt;
}

int get_int(const Node *root, const std::string &path, int dflt) {
    const Node *n = find(root, path);
    if (!n) return dflt;
    std::string t = trim(n->text);
    if (t.empty()) return dflt;
    char *end = nullptr;
    long v = std::strtol(t.c_str(), &end, 10);
    return end == t.c_str() ? dflt : (int)v;
}

bool get_bool(const Node *root, const std::string &path, bool dflt) {
    const Node *n = find(root, path);
    if (!n) return dflt;
    std::string t = trim(n->text);
    if (t == "true" || t == "1") return true;
    if (t == "false" || t == "0") return false;
    return dflt;
}

void merge_vxd(const Node *vxd_root, Node *base_root) {
    const Node *vxd = vxd_root->child("VXD");
    if (!vxd) vxd = vxd_root;
    for (auto &c : vxd->children) {
        const std::string *rep = c->attr("replace");
        if (!rep || rep->empty()) continue;
        Node *dst = find_or_create(base_root, *rep);
        std::string keep = dst->name;
        auto copy = c->clone();
        dst->attrs = copy->attrs;
        dst->text = copy->text;
        dst->children = std::move(copy->children);
        dst->name = keep;
    }
}

}  // namespace xml
}  // namespace vx3g
