"""GLSL SDF snippets beyond the reference's four shipped ones, for the tests of
the run-time compiled path (pt_glsl_translate + NVRTC).  Each has a hand
restatement in C in oracle/user_sdfs.c under the function names given here.

They use what scene authors write: helper functions with in/out parameters,
file-scope constants, swizzles (.xz, rgba), vector-scalar arithmetic, and the
built-ins length, sin, tan, asin, atan (one and two arguments), exp2, log2,
round, abs, max, min, mod, floor, clamp.
"""

TORUS = """
// Torus with a ripple; material by side of the ring.
const float R = 0.8;

float sdTorus(in vec3 p, vec2 t, out float ring)
{
    vec2 q = vec2(length(p.xz) - t.x, p.y);
    ring = q.x;
    return length(q) - t.y;
}

float sdf(vec3 p)
{
    float ring;
    float d = sdTorus(p, vec2(R, .25), ring);
    return d + 0.02 * sin(8.0 * p.x) * sin(8. * p.z);
}

float sdfmaterial(vec3 p)
{
    float ring;
    sdTorus(p, vec2(R, 0.25), ring);
    return ring > 0.0 ? 2.0 : 3.0;
}
"""

LATTICE = """
/* Rounded cubes on a lattice, clipped to a box. */
float sdBox(vec3 p, vec3 b)
{
    vec3 q = abs(p) - b;
    return length(max(q, 0.0)) + min(max(q.x, max(q.g, q.b)), 0.0);
}

float sdf(vec3 p)
{
    vec3 c = vec3(0.6);
    vec3 r = mod(p + 0.5 * c, c) - 0.5 * c;
    return max(sdBox(r, vec3(0.18)) - 0.04, sdBox(p, vec3(0.9)));
}

float sdfmaterial(vec3 p)
{
    return floor(clamp(p.y + 1.0, 0.0, 1.5)) + 1.0;
}
"""

SPIRAL = """
// A ring twisted by its polar angle; inverse and binary-log built-ins.
float sdf(vec3 p)
{
    float a = atan(p.z, p.x);
    float r = length(p.xz);
    float twist = 0.25 * sin(3.0 * a + 2.0 * p.y);
    vec2 q = vec2(r - 0.7 - 0.1 * twist, p.y);
    float k = exp2(-2.0) + 0.01 * log2(1.0 + r);
    return length(q) - 0.2 - k * 0.1 + 0.02 * asin(clamp(p.y, -1.0, 1.0)) + 0.001 * tan(0.3 * p.y);
}

float sdfmaterial(vec3 p)
{
    return round(atan(p.x) + 2.0);
}
"""

# name -> (GLSL, C function for sdf, C function for sdfmaterial)
SNIPPETS = {
    "torus": (TORUS, "user_torus_sdf", "user_torus_material"),
    "lattice": (LATTICE, "user_lattice_sdf", "user_lattice_material"),
    "spiral": (SPIRAL, "user_spiral_sdf", "user_spiral_material"),
}


def generated_params(text: str):
    """(kind, parameters) of a text pt_scene_generate wrote (oracle.generated_params)."""
    from oracle import oracle

    return oracle.generated_params(text)


def set_generated(text: str):
    """Sets the restatement of a generated snippet (oracle.set_generated)."""
    from oracle import oracle

    return oracle.set_generated(text)
