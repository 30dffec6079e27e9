// Minimal stand-in for SpaceLand's <sl/external_array.hpp>: the symvox
// sources include it but use nothing from it (oracle build only).
#pragma once
#include <sl/cstdint.hpp>
