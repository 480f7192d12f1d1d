/* Stand-in for the version header that the reference's CMake build generates from
 * crnlib/crn_version.h.in. Only used when compiling the reference sources as the oracle. */
#pragma once
#define CRN_VERSION_STR "0.0.0-oracle"
#define CRN_VERSION_NUMBER 0
#define CRN_VERSION_MAJOR 0
#define CRN_VERSION_MINOR 0
#define CRN_VERSION_PATCH 0
