// Forwards to the shared geogram shim (test infrastructure only).
#pragma once
#include "../../geo_shim.h"
