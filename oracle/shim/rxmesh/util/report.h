// Empty stand-in for the reference's report header.  The reference's
// apps/VertexNormal/vertex_normal_ref.h includes it but uses nothing from it;
// this lets oracle/Makefile compile that serial reference from its own source.
#pragma once
