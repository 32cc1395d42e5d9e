// Host-only stand-in for the few boost::filesystem names the reference headers
// mention (oracle reference build only; no file-system work happens through it).
#pragma once
#include <string>
namespace boost { namespace filesystem {
struct path {
    std::string s;
    path() {}
    path(const char *c) : s(c) {}
    path(const std::string &c) : s(c) {}
    std::string string() const { return s; }
    const char *c_str() const { return s.c_str(); }
    path filename() const { return *this; }
    path extension() const { return *this; }
};
} }
