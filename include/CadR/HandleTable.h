// CadR/HandleTable.h - the reference's per-class header name (src/CadR/HandleTable.h); the
// facade declares HandleTable in CadR/DataStorage.h.
#pragma once

#include "DataStorage.h"
