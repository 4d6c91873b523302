// Host shim: every ModernGPU header the reference includes maps to one file.
#pragma once
#include "mgpu_host.hxx"
