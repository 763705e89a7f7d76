// CadR/FrameInfo.h - the reference's per-class header name (src/CadR/FrameInfo.h); the
// facade declares FrameInfo in CadR/Renderer.h.
#pragma once

#include "Renderer.h"
