// ORACLE harness include shim.  hash_dag_factory.cpp includes the GL-interop
// tracer wrapper only for DAGInfo; the harness builds no tracer host code, so
// this stand-in provides DAGInfo alone.
#pragma once
#include "dag_info.h"
