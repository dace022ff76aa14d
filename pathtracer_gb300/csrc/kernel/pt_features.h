// pt_features.h — compiled variants of the path kernels by primitive class.
#pragma once

// Primitive classes a kernel variant handles.  A variant without a class
// must only see scenes that have none of it; the arithmetic of the classes
// it keeps is unchanged, so every variant gives the same bits.
enum : int {
    PT_FEAT_BOX = 1,
    PT_FEAT_LENS = 2,
    PT_FEAT_CYCLIDE = 4,
    PT_FEAT_SDF = 8,
    PT_FEAT_ANALYTIC = PT_FEAT_BOX | PT_FEAT_LENS | PT_FEAT_CYCLIDE,
    PT_FEAT_ALL = PT_FEAT_ANALYTIC | PT_FEAT_SDF
};

// The smallest compiled variant (0, BOX, ANALYTIC, ALL) covering a scene
// with the given object counts.
inline int pt_feature_variant(const int n[7]) {
    if (n[5] > 0) return PT_FEAT_ALL;
    if (n[3] > 0 || n[4] > 0) return PT_FEAT_ANALYTIC;
    if (n[2] > 0) return PT_FEAT_BOX;
    return 0;
}
inline int pt_variant_union(int a, int b) {
    const int m = a | b;
    if (m & PT_FEAT_SDF) return PT_FEAT_ALL;
    if (m & (PT_FEAT_LENS | PT_FEAT_CYCLIDE)) return PT_FEAT_ANALYTIC;
    return m;
}
