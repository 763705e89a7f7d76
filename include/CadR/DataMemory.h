// CadR/DataMemory.h - the reference's per-class header name (src/CadR/DataMemory.h); the
// facade declares DataMemory in CadR/DataStorage.h.
#pragma once

#include "DataStorage.h"
