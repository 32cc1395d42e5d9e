// vx3g_xml.h -- a small DOM for VXA/VXD documents and the VXD merge.
//
// The reference reads VXA/VXD files with boost::property_tree (merge) and
// tinyxml/CXML_Rip (import).  This header provides the pieces the host side
// needs without Boost: an element tree with attributes, text and CDATA, a
// path lookup "VXA.Simulator.Integration.DtFrac" with property_tree's
// get<T>(path, default) meaning, and ctool::ptree_merge's VXD rule
// (src/Utils/ctool.h:49-57): every child of <VXD> that carries
// replace="A.B.C" replaces the node at that path in the base tree.
#pragma once

#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

namespace vx3g {
namespace xml {

struct Node {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::string text;  // concatenated character data and CDATA of this element
    std::vector<std::unique_ptr<Node>> children;

    const Node *child(const std::string &n) const {
        for (auto &c : children)
            if (c->name == n) return c.get();
        return nullptr;
    }
    Node *child(const std::string &n) {
        for (auto &c : children)
            if (c->name == n) return c.get();
        return nullptr;
    }
    std::vector<const Node *> all(const std::string &n) const {
        std::vector<const Node *> out;
        for (auto &c : children)
            if (c->name == n) out.push_back(c.get());
        return out;
    }
    const std::string *attr(const std::string &n) const {
        for (auto &a : attrs)
            if (a.first == n) return &a.second;
        return nullptr;
    }
    std::unique_ptr<Node> clone() const;
};

// Parses a document; returns a synthetic root whose children are the top-level
// elements.  Throws std::runtime_error on malformed input.
std::unique_ptr<Node> parse(const std::string &text);
std::unique_ptr<Node> parse_file(const std::string &path);

// Node at a dotted path below root (the first path element names a child of
// root), or nullptr.
const Node *find(const Node *root, const std::string &path);
Node *find_or_create(Node *root, const std::string &path);

// property_tree-like typed reads of a node's trimmed text
bool get_double(const Node *root, const std::string &path, double *out);
double get_double(const Node *root, const std::string &path, double dflt);
int get_int(const Node *root, const std::string &path, int dflt);
bool get_bool(const Node *root, const std::string &path, bool dflt);

// ctool::ptree_merge: apply the replace="path" children of <VXD> to base.
void merge_vxd(const Node *vxd_root, Node *base_root);

std::string trim(const std::string &s);

}  // namespace xml
}  // namespace vx3g
