// Strong definition of fnv_hash(unsigned, unsigned) that forwards to the
// reference's own Normal_APHash (rankSelectQuotientFilter/CPU_version/
// RSQF.cpp:168-183, the hash the reference GPU SQF uses at
// quotientFilter.cu:268).  oracle/build_ref.sh links it against a copy of the
// CPU_version object whose fnv_hash was made weak, so the reference's own
// insertItem/mayContain run with the GPU hash.  Test infrastructure only.
unsigned int Normal_APHash(unsigned int value, unsigned int maxHashValue);
unsigned int fnv_hash(unsigned int value, unsigned int tableSize)
{
    return Normal_APHash(value, tableSize);
}
