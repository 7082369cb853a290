# CMake package of the GB300 GMlib, in place of the reference's installed
# GMlibConfig.cmake (reference CMakeLists.txt:137-150): a caller's
#   find_package(GMlib 3 REQUIRED)
#   target_link_libraries(app GM.3)        # or ${GMlib_LIBRARIES}
#   include_directories(${GMlib_INCLUDE_DIRS})
#   compile_cl(body)                       # body.cl -> body.h (char *body)
# works unchanged with CMAKE_PREFIX_PATH (or GMlib_DIR) pointing at this
# directory.  GM.3 is the shared library gmlib_gb300/libgmlib3.so (CUDA
# runtime linked in, NVRTC from the CUDA toolkit) built by
# `python -m gmlib_gb300.build`, which also builds the cl2h tool used here.

get_filename_component(_gml_pkg "${CMAKE_CURRENT_LIST_DIR}/.." ABSOLUTE)
get_filename_component(_gml_root "${_gml_pkg}/.." ABSOLUTE)

if(NOT EXISTS "${_gml_pkg}/libgmlib3.so")
  set(GMlib_FOUND FALSE)
  set(GMlib_NOT_FOUND_MESSAGE
      "${_gml_pkg}/libgmlib3.so is missing: run python -m gmlib_gb300.build")
  return()
endif()

if(NOT TARGET GM.3)
  add_library(GM.3 SHARED IMPORTED)
  set_target_properties(GM.3 PROPERTIES
    IMPORTED_LOCATION "${_gml_pkg}/libgmlib3.so"
    INTERFACE_INCLUDE_DIRECTORIES "${_gml_root}/include"
    INTERFACE_LINK_LIBRARIES "m")
endif()

set(GMlib_INCLUDE_DIRS "${_gml_root}/include")
set(GMlib_LIBRARIES GM.3)
set(GMlib_CL2H "${_gml_pkg}/cl2h")
set(GMlib_FOUND TRUE)

# the reference's macro (CMakeLists.txt:39-46): <basename>.cl in the current
# source directory -> <basename>.h in the current binary directory, declaring
# char *<basename>
macro(compile_cl basename)
  add_custom_command(
    OUTPUT ${CMAKE_CURRENT_BINARY_DIR}/${basename}.h
    COMMAND ${GMlib_CL2H} ${CMAKE_CURRENT_SOURCE_DIR}/${basename}.cl
            ${CMAKE_CURRENT_BINARY_DIR}/${basename}.h ${basename}
    DEPENDS ${CMAKE_CURRENT_SOURCE_DIR}/${basename}.cl)
endmacro(compile_cl)
