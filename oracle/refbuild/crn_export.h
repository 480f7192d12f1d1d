/* Stand-in for the export header that the reference's CMake build generates
 * (generate_export_header in crnlib/CMakeLists.txt). Only used when compiling the
 * reference sources as the test oracle; the symbol visibility macros are all it needs. */
#pragma once
#define CRN_EXPORT __attribute__((visibility("default")))
#define CRN_NO_EXPORT __attribute__((visibility("hidden")))
#define CRN_DEPRECATED __attribute__((__deprecated__))
#define CRN_DEPRECATED_EXPORT CRN_EXPORT CRN_DEPRECATED
#define CRN_DEPRECATED_NO_EXPORT CRN_NO_EXPORT CRN_DEPRECATED
