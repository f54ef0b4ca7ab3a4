// Stand-in for the version header the reference's CMake build generates
// (version.cmake); Utils.cpp prints these.
#ifndef A2C_REF_SHIM_VERSION_H
#define A2C_REF_SHIM_VERSION_H
#define GIT_REV "N/A"
#define GIT_TAG "N/A"
#define GIT_BRANCH "N/A"
#endif
