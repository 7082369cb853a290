// A double-precision tetrahedron field read into a local value (checks
// that an FP64 datatype compiles and launches; nothing is written).
double twice = 2.0 * Wide;
