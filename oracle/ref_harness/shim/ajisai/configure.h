/* Stand-in for the CMake-generated ajisai/configure.h: the reference's
 * template only carries target switches, none of which the harness needs. */
#pragma once
#define AJISAI_TARGET_UNIX
