// The tetrahedron's four node indices, converted to floats.
Cel = convert_float4(TetVer);
