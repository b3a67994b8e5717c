#pragma once
typedef int MPI_Comm;
