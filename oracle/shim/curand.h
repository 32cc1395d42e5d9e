// Host-only stand-in (oracle reference build only).
#pragma once
