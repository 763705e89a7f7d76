// CadR/MatrixList.h - the reference's per-class header name (src/CadR/MatrixList.h); the
// facade declares MatrixList in CadR/Renderer.h.
#pragma once

#include "Renderer.h"
