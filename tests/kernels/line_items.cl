// Reads and rewrites every item of 2- and 4-item lines (float4, int4,
// double2): the generated prologue and epilogue move such 32- and 64-byte
// lines with 32-byte loads and stores.
{
   float4 t0 = A[0], t1 = A[1], t2 = A[2], t3 = A[3];
   A[0] = t1 + t2;
   A[1] = t2 - t0;
   A[2] = t3 + t3;
   A[3] = t0 - t1;
   int4 u0 = C[0], u1 = C[1], u2 = C[2], u3 = C[3];
   C[0] = u3;
   C[1] = u2 + u0;
   C[2] = u1 - u3;
   C[3] = u0;
   float4 b0 = B[0];
   B[0] = B[1];
   B[1] = b0 + b0;
   double2 d0 = D[0];
   D[0] = D[1] + d0;
   D[1] = d0 - D[1];
}
