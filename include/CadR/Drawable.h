// CadR/Drawable.h - the reference's per-class header name (src/CadR/Drawable.h); the
// facade declares Drawable in CadR/Renderer.h.
#pragma once

#include "Renderer.h"
