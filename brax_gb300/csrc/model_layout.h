// Packed model descriptor: one array of 32-bit words (int32 or float32 bit
// patterns).  The first BXM_HEADER_WORDS words are the header below; every
// BXM_O_* entry holds the word offset of an array inside the same blob.
// brax_gb300/model_pack.py writes this layout; the kernels read it from shared
// memory.  Field meanings follow brax's System (brax/base.py:415-540).
#pragma once

#define BXM_MAGIC 0x42584D31  // "BXM1"
#define BXM_VERSION 1

enum BxmHeader {
  BXM_H_MAGIC = 0,
  BXM_H_VERSION,
  BXM_H_WORDS,        // total words in the blob
  BXM_H_NL,           // links
  BXM_H_NQ,
  BXM_H_NV,
  BXM_H_NU,
  BXM_H_NCON,         // contact slots
  BXM_H_NLIM,         // limit rows (0 when no dof is limited)
  BXM_H_M,            // constraint rows = 4*ncon + nlim
  BXM_H_NLEVEL,       // tree depth levels
  BXM_H_NS_ITERS,     // matrix_inv_iterations
  BXM_H_PG_ITERS,     // solver_iterations
  BXM_H_PG_MAXLS,     // solver_maxls
  BXM_H_NROOT,
  BXM_H_DT,           // float
  BXM_H_GX,           // float gravity
  BXM_H_GY,
  BXM_H_GZ,
  BXM_H_PG_TOL,       // float (jaxopt default 1e-3)
  BXM_H_FLUID,        // 1 when viscosity or density is nonzero (System.enable_fluid)
  BXM_H_VISC,         // float fluid viscosity
  BXM_H_DENS,         // float fluid density
  // int arrays
  BXM_O_LINK_PARENT,  // [nl]
  BXM_O_LINK_TYPE,    // [nl] 0 = free, 1/2/3 = stacked hinge/slide dofs
  BXM_O_LINK_QADR,    // [nl]
  BXM_O_LINK_DADR,    // [nl]
  BXM_O_LINK_ROOT,    // [nl]
  BXM_O_LEVEL_START,  // [nlevel + 1]
  BXM_O_LEVEL_LINKS,  // [nl] links in level order
  BXM_O_CHILD_START,  // [nl + 1]
  BXM_O_CHILD_IDX,    // [nl]
  BXM_O_DOF_LINK,     // [nv]
  BXM_O_LINK_ANC,     // [nl * 2] 64-bit mask of the dofs of ancestor-or-self links
  BXM_O_LIM_DOF,      // [nlim]
  BXM_O_LIM_QADR,     // [nlim]
  BXM_O_ACT_QID,      // [nu]
  BXM_O_ACT_QDID,     // [nu]
  BXM_O_CON_KIND,     // [ncon]
  BXM_O_CON_SUB,      // [ncon]
  BXM_O_CON_LA,       // [ncon] link of geom1 (-1 = world)
  BXM_O_CON_LB,       // [ncon] link of geom2
  // float arrays
  BXM_O_LT_POS,       // [nl*3] link.transform
  BXM_O_LT_ROT,       // [nl*4]
  BXM_O_LJ_POS,       // [nl*3] link.joint (rotation is identity)
  BXM_O_LI_POS,       // [nl*3] link.inertia.transform
  BXM_O_LI_ROT,       // [nl*4]
  BXM_O_LI_I,         // [nl*9]
  BXM_O_LI_MASS,      // [nl]
  BXM_O_L_INVW,       // [nl]
  BXM_O_ROOT_MASS,    // [nl] mass of the link's tree
  BXM_O_D_ANG,        // [nv*3] dof.motion
  BXM_O_D_VEL,        // [nv*3]
  BXM_O_D_ARM,        // [nv]
  BXM_O_D_STIFF,      // [nv]
  BXM_O_D_DAMP,       // [nv]
  BXM_O_D_INVW,       // [nv]
  BXM_O_LIM_LO,       // [nlim]
  BXM_O_LIM_HI,       // [nlim]
  BXM_O_LIM_INVW,     // [nlim]
  BXM_O_LIM_SOLP,     // [nlim*7]
  BXM_O_ACT_CR,       // [nu*2]
  BXM_O_ACT_FR,       // [nu*2]
  BXM_O_ACT_GAIN,     // [nu]
  BXM_O_ACT_GEAR,     // [nu]
  BXM_O_ACT_BQ,       // [nu]
  BXM_O_ACT_BQD,      // [nu]
  BXM_O_CON_G1POS,    // [ncon*3] geom1 pose in its link frame
  BXM_O_CON_G1QUAT,   // [ncon*4]
  BXM_O_CON_G1SIZE,   // [ncon*3]
  BXM_O_CON_G2POS,    // [ncon*3]
  BXM_O_CON_G2QUAT,   // [ncon*4]
  BXM_O_CON_G2SIZE,   // [ncon*3]
  BXM_O_CON_FRIC,     // [ncon] sliding friction
  BXM_O_CON_INVW,     // [ncon] invweight[la]*(la>-1) + invweight[lb]
  BXM_O_CON_SOLP,     // [ncon*7] solref + solimp
  BXM_O_LI_BOX,       // [nl*3] inertia-equivalent box of each link (brax/fluid.py:71-76)
  BXM_HEADER_WORDS = 128
};

// collision kinds (match brax_gb300/system.py CON_*)
#define BXM_CON_PLANE_SPHERE 0
#define BXM_CON_PLANE_CAPSULE 1
#define BXM_CON_PLANE_BOX 2
#define BXM_CON_SPHERE_SPHERE 3
#define BXM_CON_SPHERE_CAPSULE 4
#define BXM_CON_CAPSULE_CAPSULE 5
