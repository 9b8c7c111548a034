// Backend list line for libCEED's backends/ceed-backend-list.h (include this file from it).
// CEED_BACKEND(registration function, number of resources, resource prefix)
CEED_BACKEND(CeedRegister_B200, 1, "/gpu/cuda/b200")
