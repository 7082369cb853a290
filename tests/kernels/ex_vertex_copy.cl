// The vertex coordinates copied into a vertex field (a direct read and a
// direct write per vertex).
Pts = VerCrd;
