/* Quality of a quadratic (P2) tetrahedron, the measure of the reference's
   P2Quality example written independently: the product of
     the Jacobian ratio   min / max of the cubic Bernstein coefficients of
                          det J over the control net,
     the shape factor     2 sqrt(6) V2 / (L S),
     the volume ratio     min(V1, V2) / max(V1, V2),
   with L the longest edge measured through its mid node, S the summed
   |cross| of the 16 triangles splitting the faces at their mid nodes, V1 six
   times the straight volume and V2 six times the volume those triangles
   enclose.  VerCrd[4]: vertices; MidCrd[6]: mid-edge nodes of the local
   edges (0,1) (1,2) (2,0) (3,0) (3,1) (3,2), read through TetEdg. */
{
   const int ea[6] = {0, 1, 2, 3, 3, 3}, eb[6] = {1, 2, 0, 0, 1, 2};
   const int fa[4] = {1, 0, 0, 0}, fb[4] = {2, 3, 1, 2}, fc[4] = {3, 2, 3, 1};
   const int ei[16] = {-1, 0, 2, 3,  0, -1, 1, 4,  2, 1, -1, 5,  3, 4, 5, -1};
   float4 ctl[16], d[12], o = VerCrd[0];
   float L = 0.f, S = 0.f, V1, V2 = 0.f, jmin = 0.f, jmax = 0.f, bin[64];
   int i, j, k, f;

   for(i=0;i<6;i++)
      L = fmax(L, fast_distance(VerCrd[ ea[i] ], MidCrd[i]) + fast_distance(MidCrd[i], VerCrd[ eb[i] ]));

   for(f=0;f<4;f++)
   {
      float4 a = VerCrd[ fa[f] ], b = VerCrd[ fb[f] ], c = VerCrd[ fc[f] ];
      float4 ab = MidCrd[ ei[ 4*fa[f] + fb[f] ] ];
      float4 bc = MidCrd[ ei[ 4*fb[f] + fc[f] ] ];
      float4 ca = MidCrd[ ei[ 4*fc[f] + fa[f] ] ];
      float4 t[12] = {a, ab, ca,  ab, b, bc,  ca, bc, c,  ab, bc, ca};
      for(k=0;k<4;k++)
      {
         float4 p = t[3*k] - o, q = t[3*k+1] - o, r = t[3*k+2] - o;
         S += fast_length(cross(q - p, r - p));
         V2 += dot(cross(p, q), r);
      }
   }
   V1 = dot(cross(VerCrd[1] - o, VerCrd[2] - o), VerCrd[3] - o);

   /* control net: vertices on the diagonal, c_e = 2 m_e - (a + b) / 2 */
   for(i=0;i<4;i++)
      ctl[ 5*i ] = VerCrd[i];
   for(i=0;i<6;i++)
   {
      float4 c = 2.f * MidCrd[i] - .5f * (VerCrd[ ea[i] ] + VerCrd[ eb[i] ]);
      ctl[ 4*ea[i] + eb[i] ] = c;
      ctl[ 4*eb[i] + ea[i] ] = c;
   }
   /* derivative control vectors along lambda_{k+1} - lambda_0 */
   for(k=0;k<3;k++)
      for(i=0;i<4;i++)
         d[ 4*k + i ] = ctl[ 4*i + k + 1 ] - ctl[ 4*i ];

   /* fully unrolled, so that every bin index is a constant and the bins
      stay in registers */
   #pragma unroll
   for(i=0;i<64;i++)
      bin[i] = 0.f;
   #pragma unroll
   for(i=0;i<4;i++)
      #pragma unroll
      for(j=0;j<4;j++)
      {
         float4 n = cross(d[i], d[4 + j]);
         #pragma unroll
         for(k=0;k<4;k++)
         {
            int x = min(i, min(j, k)), z = max(i, max(j, k)), y = i + j + k - x - z;
            bin[ 16*x + 4*y + z ] += dot(n, d[8 + k]);
         }
      }
   f = 1;
   #pragma unroll
   for(i=0;i<4;i++)
      #pragma unroll
      for(j=i;j<4;j++)
         #pragma unroll
         for(k=j;k<4;k++)
         {
            float w = (i == k) ? 8.f : (i == j || j == k) ? 8.f / 3.f : 4.f / 3.f;
            float nj = w * bin[ 16*i + 4*j + k ];
            jmin = f ? nj : fmin(jmin, nj);
            jmax = f ? nj : fmax(jmax, nj);
            f = 0;
         }

   qal = (jmin / jmax) * ((2.f * sqrt(6.f) * V2) / (L * S)) * (fmin(V1, V2) / fmax(V1, V2));
}
