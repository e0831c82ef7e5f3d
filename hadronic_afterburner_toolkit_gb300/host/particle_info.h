// One particle of a sample (fields of the reference's particle_info,
// src/particle_info.h).
#pragma once

typedef struct {
    int monval;
    double mass;
    int baryon;
    double px, py, pz, E;
    double x, y, z, t;
    double rap_y, rap_eta, pT, phi_p;
} particle_info;
