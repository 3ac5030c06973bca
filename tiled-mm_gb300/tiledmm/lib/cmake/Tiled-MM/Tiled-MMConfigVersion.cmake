# Version of the Tiled-MM API this package provides: 2.3.1, the reference's
# (CMakeLists.txt project version).  A request is compatible when its major
# version is 2 and it asks for no more than 2.3.1 (same-major compatibility).
set(PACKAGE_VERSION "2.3.1")
if(PACKAGE_FIND_VERSION_MAJOR STREQUAL "" OR PACKAGE_FIND_VERSION_MAJOR EQUAL 2)
  if(PACKAGE_FIND_VERSION VERSION_GREATER PACKAGE_VERSION)
    set(PACKAGE_VERSION_COMPATIBLE FALSE)
  else()
    set(PACKAGE_VERSION_COMPATIBLE TRUE)
    if(PACKAGE_FIND_VERSION STREQUAL PACKAGE_VERSION)
      set(PACKAGE_VERSION_EXACT TRUE)
    endif()
  endif()
else()
  set(PACKAGE_VERSION_COMPATIBLE FALSE)
endif()
