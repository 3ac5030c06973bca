# CMake package configuration of the GB300 build of Tiled-MM.
#
# A consumer written against the reference package keeps its CMake code:
#
#   find_package(Tiled-MM REQUIRED)
#   target_link_libraries(app PRIVATE Tiled-MM::Tiled-MM)
#
# with CMAKE_PREFIX_PATH (or Tiled-MM_DIR) pointing at this package: the
# directory tiled-mm_gb300/tiledmm of the repository (or this file's own
# directory).  Tiled-MM::Tiled-MM is the in-tree shared library
# (tiled-mm_gb300/build.py builds it) with the drop-in headers <Tiled-MM/...>
# and the C ABI <tmm_c_api.h>, C++14 or later, and the TILED_MM_CUDA definition
# the reference's target exports.  No CUDA toolkit is needed to link against it:
# the CUDA runtime is linked into the library.
get_filename_component(_tmm_prefix "${CMAKE_CURRENT_LIST_DIR}/../../.." ABSOLUTE)
get_filename_component(_tmm_root "${_tmm_prefix}/../.." ABSOLUTE)
set(_tmm_lib "${_tmm_prefix}/lib/libtiledmm_gb300.so")
set(_tmm_inc "${_tmm_root}/include")

if(NOT EXISTS "${_tmm_lib}" OR NOT EXISTS "${_tmm_inc}/Tiled-MM/tiled_mm.hpp")
  set(Tiled-MM_FOUND FALSE)
  set(Tiled-MM_NOT_FOUND_MESSAGE
      "Tiled-MM (GB300): ${_tmm_lib} is missing; build it with `python tiled-mm_gb300/build.py`")
  return()
endif()

if(NOT TARGET Tiled-MM::Tiled-MM)
  add_library(Tiled-MM::Tiled-MM SHARED IMPORTED)
  set_target_properties(Tiled-MM::Tiled-MM PROPERTIES
    IMPORTED_LOCATION "${_tmm_lib}"
    IMPORTED_SONAME "libtiledmm_gb300.so"
    INTERFACE_INCLUDE_DIRECTORIES "${_tmm_inc}"
    INTERFACE_COMPILE_DEFINITIONS "TILED_MM_CUDA"
    INTERFACE_COMPILE_FEATURES "cxx_std_14")
endif()

set(Tiled-MM_INCLUDE_DIRS "${_tmm_inc}")
set(Tiled-MM_LIBRARIES Tiled-MM::Tiled-MM)
unset(_tmm_prefix)
unset(_tmm_root)
unset(_tmm_lib)
unset(_tmm_inc)
