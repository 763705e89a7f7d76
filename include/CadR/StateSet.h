// CadR/StateSet.h - the reference's per-class header name (src/CadR/StateSet.h); the
// facade declares StateSet in CadR/Renderer.h.
#pragma once

#include "Renderer.h"
