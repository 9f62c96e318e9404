/* host stand-in: only the type names used in declarations */
#pragma once
typedef struct { unsigned int d[12]; } curandState;
