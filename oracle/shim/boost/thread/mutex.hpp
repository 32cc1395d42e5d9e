// Host-only stand-in (oracle reference build only; single-threaded).
#pragma once
namespace boost { struct mutex { void lock() {} void unlock() {} }; }
