// Per vertex: the ball sum of a tetrahedron field, times GmlPar->res over
// the degree, stored in both items of the vertex field.
{
   float4 acc = (float4)(0.0f);
   for(int k = 0; k < MidDegMax; k++)
      acc += Mid[k];
   Sol[0] = GmlPar->res * acc / MidDeg;
   Sol[1] = GmlPar->res * acc / MidDeg;
}
