// Export.h -- FASTNOISE_API for the C++ layer of the GB300 backend.
//
// Same macro name as the reference's include/FastNoise/Utility/Export.h:1-17, so code that
// tests or uses it compiles unchanged.  The C++ layer is header-only over the C-ABI of
// libfastnoise_gb300.so; the macro marks the exported C functions it calls.
#pragma once

#ifndef FASTNOISE_API
#if defined(_WIN32)
#define FASTNOISE_API __declspec(dllimport)
#else
#define FASTNOISE_API __attribute__((visibility("default")))
#endif
#endif
