// CadR/PrimitiveSet.h - the reference's per-class header name (src/CadR/PrimitiveSet.h); the
// facade declares PrimitiveSet in CadR/Renderer.h.
#pragma once

#include "Renderer.h"
