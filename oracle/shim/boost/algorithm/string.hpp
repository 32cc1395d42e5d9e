// Host-only stand-in (oracle reference build only).
#pragma once
#include <string>
namespace boost { inline void to_upper(std::string &) {} }
