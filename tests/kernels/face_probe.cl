// Which triangles a tet's four faces are: a triangle field holding index + 1,
// read through the tet -> triangle downlink.
{
   TetTri = (float4)(TriNum[0], TriNum[1], TriNum[2], TriNum[3]);
}
