/* Included by the reference's src/Molecule.h:4; nothing from it is used. */
#pragma once
