// CadR/StagingData.h - the reference's per-class header name (src/CadR/StagingData.h); the
// facade declares StagingData in CadR/DataStorage.h.
#pragma once

#include "DataStorage.h"
