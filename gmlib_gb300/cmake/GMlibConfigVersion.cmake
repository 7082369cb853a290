# Version of the GB300 GMlib package: 3.41, the reference's version
# (reference CMakeLists.txt:3-4), compatible with requests of the same major
# version as write_basic_package_version_file(... SameMajorVersion) gives.
set(PACKAGE_VERSION "3.41")
if(PACKAGE_FIND_VERSION_MAJOR AND NOT PACKAGE_FIND_VERSION_MAJOR STREQUAL "3")
  set(PACKAGE_VERSION_COMPATIBLE FALSE)
elseif(PACKAGE_FIND_VERSION VERSION_GREATER PACKAGE_VERSION)
  set(PACKAGE_VERSION_COMPATIBLE FALSE)
else()
  set(PACKAGE_VERSION_COMPATIBLE TRUE)
  if(PACKAGE_FIND_VERSION STREQUAL PACKAGE_VERSION)
    set(PACKAGE_VERSION_EXACT TRUE)
  endif()
endif()
