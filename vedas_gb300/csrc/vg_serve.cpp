// The serving loop is header-only (vg_serve.h); this unit anchors it in the build.
#include "vg_serve.h"
