// CadR/Geometry.h - the reference's per-class header name (src/CadR/Geometry.h); the
// facade declares Geometry in CadR/Renderer.h.
#pragma once

#include "Renderer.h"
