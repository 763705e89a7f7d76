// CadR/DataAllocation.h - the reference's per-class header name (src/CadR/DataAllocation.h); the
// facade declares DataAllocation in CadR/DataStorage.h.
#pragma once

#include "DataStorage.h"
