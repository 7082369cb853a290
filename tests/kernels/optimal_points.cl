// For each face of the tetrahedron, the apex of a regular tetrahedron built
// on it: face centroid + unit normal * 0.816496 * longest face edge.
{
   const int fv[4][3] = { {1,2,3}, {0,2,3}, {1,0,3}, {1,2,0} };
   float4 ctr, nrm, u, v;
   float  h;
   int    f;

   for(f=0;f<4;f++)
   {
      float4 a = VerCrd[ fv[f][0] ], b = VerCrd[ fv[f][1] ], c = VerCrd[ fv[f][2] ];
      h   = max(max(dot(a - b, a - b), dot(a - c, a - c)), dot(b - c, b - c));
      h   = 0.816496 * sqrt(h);
      ctr = (a + b + c) * (float4)(1./3.);
      u   = (f == 0) ? VerCrd[1] - VerCrd[3] : (f == 1) ? VerCrd[2] - VerCrd[3]
          : (f == 2) ? VerCrd[0] - VerCrd[3] : VerCrd[1] - VerCrd[2];
      v   = (f == 0) ? VerCrd[2] - VerCrd[3] : (f == 1) ? VerCrd[0] - VerCrd[3]
          : (f == 2) ? VerCrd[1] - VerCrd[3] : VerCrd[0] - VerCrd[2];
      nrm = fast_normalize(cross(u, v)) * (float4)(h);
      OptCrd[f] = ctr + nrm;
   }
}
