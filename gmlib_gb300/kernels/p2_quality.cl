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
   edges (0,1) (1,2) (2,0) (3,0) (3,1) (3,2), read through the tet -> edge
   link.  Scalar x, y, z arithmetic: the unused w lane of the float4 nodes is
   never computed, and fewer live registers leave room for more warps. */
{
   const int ea[6] = {0, 1, 2, 3, 3, 3}, eb[6] = {1, 2, 0, 0, 1, 2};
   const int fa[4] = {1, 0, 0, 0}, fb[4] = {2, 3, 1, 2}, fc[4] = {3, 2, 3, 1};
   const int ei[16] = {-1, 0, 2, 3,  0, -1, 1, 4,  2, 1, -1, 5,  3, 4, 5, -1};
   /* nodes relative to vertex 0: 0..3 vertices, 4..9 mid-edge nodes */
   float nx[10], ny[10], nz[10];
   float L = 0.f, S = 0.f, V1, V2 = 0.f, jmin = 0.f, jmax = 0.f, bin[64];
   float dx[12], dy[12], dz[12];
   int i, j, k, f;

   #pragma unroll
   for(i=0;i<4;i++)
   {
      nx[i] = VerCrd[i].x - VerCrd[0].x;
      ny[i] = VerCrd[i].y - VerCrd[0].y;
      nz[i] = VerCrd[i].z - VerCrd[0].z;
   }
   #pragma unroll
   for(i=0;i<6;i++)
   {
      nx[4+i] = MidCrd[i].x - VerCrd[0].x;
      ny[4+i] = MidCrd[i].y - VerCrd[0].y;
      nz[4+i] = MidCrd[i].z - VerCrd[0].z;
   }

   /* longest edge through its mid node */
   #pragma unroll
   for(i=0;i<6;i++)
   {
      const float ax = nx[4+i] - nx[ ea[i] ], ay = ny[4+i] - ny[ ea[i] ], az = nz[4+i] - nz[ ea[i] ];
      const float bx = nx[ eb[i] ] - nx[4+i], by = ny[ eb[i] ] - ny[4+i], bz = nz[ eb[i] ] - nz[4+i];
      L = fmax(L, sqrt(ax*ax + ay*ay + az*az) + sqrt(bx*bx + by*by + bz*bz));
   }

   /* the 16 face triangles: |cross| summed, and their enclosed volume */
   #pragma unroll
   for(f=0;f<4;f++)
   {
      const int a = fa[f], b = fb[f], c = fc[f];
      const int ab = 4 + ei[4*a + b], bc = 4 + ei[4*b + c], ca = 4 + ei[4*c + a];
      const int t[12] = {a, ab, ca,  ab, b, bc,  ca, bc, c,  ab, bc, ca};
      #pragma unroll
      for(k=0;k<4;k++)
      {
         const int p = t[3*k], q = t[3*k+1], r = t[3*k+2];
         const float ux = nx[q] - nx[p], uy = ny[q] - ny[p], uz = nz[q] - nz[p];
         const float vx = nx[r] - nx[p], vy = ny[r] - ny[p], vz = nz[r] - nz[p];
         const float cx = uy*vz - uz*vy, cy = uz*vx - ux*vz, cz = ux*vy - uy*vx;
         S += sqrt(cx*cx + cy*cy + cz*cz);
         V2 += nx[p] * (ny[q]*nz[r] - nz[q]*ny[r])
             + ny[p] * (nz[q]*nx[r] - nx[q]*nz[r])
             + nz[p] * (nx[q]*ny[r] - ny[q]*nx[r]);
      }
   }
   V1 = nx[1] * (ny[2]*nz[3] - nz[2]*ny[3]) + ny[1] * (nz[2]*nx[3] - nx[2]*nz[3])
      + nz[1] * (nx[2]*ny[3] - ny[2]*nx[3]);

   /* mid-edge nodes to control points, c_e = 2 m_e - (a + b) / 2 */
   #pragma unroll
   for(i=0;i<6;i++)
   {
      nx[4+i] = 2.f * nx[4+i] - .5f * (nx[ ea[i] ] + nx[ eb[i] ]);
      ny[4+i] = 2.f * ny[4+i] - .5f * (ny[ ea[i] ] + ny[ eb[i] ]);
      nz[4+i] = 2.f * nz[4+i] - .5f * (nz[ ea[i] ] + nz[ eb[i] ]);
   }
   /* derivative control vectors along lambda_{k+1} - lambda_0: point (g, k+1)
      minus point (g, 0) of the net (a vertex when both indices agree) */
   #pragma unroll
   for(k=0;k<3;k++)
      #pragma unroll
      for(i=0;i<4;i++)
      {
         const int p = i == k + 1 ? i : 4 + ei[4*i + k + 1];
         const int q = i == 0 ? 0 : 4 + ei[4*i];
         dx[4*k + i] = nx[p] - nx[q];
         dy[4*k + i] = ny[p] - ny[q];
         dz[4*k + i] = nz[p] - nz[q];
      }

   /* cubic Bernstein coefficients of det J: the triple products of one
      vector per direction, summed over the orderings of each multi-index */
   #pragma unroll
   for(i=0;i<64;i++)
      bin[i] = 0.f;
   #pragma unroll
   for(i=0;i<4;i++)
      #pragma unroll
      for(j=0;j<4;j++)
      {
         const float cx = dy[i]*dz[4+j] - dz[i]*dy[4+j];
         const float cy = dz[i]*dx[4+j] - dx[i]*dz[4+j];
         const float cz = dx[i]*dy[4+j] - dy[i]*dx[4+j];
         #pragma unroll
         for(k=0;k<4;k++)
         {
            const int x = min(i, min(j, k)), z = max(i, max(j, k)), y = i + j + k - x - z;
            bin[ 16*x + 4*y + z ] += cx*dx[8+k] + cy*dy[8+k] + cz*dz[8+k];
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
            const float w = (i == k) ? 8.f : (i == j || j == k) ? 8.f / 3.f : 4.f / 3.f;
            const float nj = w * bin[ 16*i + 4*j + k ];
            jmin = f ? nj : fmin(jmin, nj);
            jmax = f ? nj : fmax(jmax, nj);
            f = 0;
         }

   qal = (jmin / jmax) * ((2.f * sqrt(6.f) * V2) / (L * S)) * (fmin(V1, V2) / fmax(V1, V2));
}
