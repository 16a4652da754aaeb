// Compile-time stand-in for CSXCAD's ContinuousStructure.h: the
// declarations the openEMS engine / operator headers name, so that the
// Engine_CUDA / Operator_CUDA glue can be compiled against those headers
// without CSXCAD.  Nothing here is called.
#pragma once
#include <string>
#include <vector>

enum CoordinateSystem { CARTESIAN, CYLINDRICAL, UNDEFINED_CS };

class CSPrimitives;
class CSPrimBox;
class CSPrimCurve;
class CSRectGrid;
class CSBackgroundMaterial;
class CSPropLumpedElement;
class CSPropMaterial;
class CSPropLorentzMaterial;
class CSPropDebyeMaterial;
class CSPropExcitation;
class TiXmlElement;

class CSProperties {
public:
    enum PropertyType {
        ANY = 0xfff, UNKNOWN = 0x001, MATERIAL = 0x002, METAL = 0x004, EXCITATION = 0x008, PROBEBOX = 0x010,
        RESBOX = 0x020, DUMPBOX = 0x040, DISPERSIVEMATERIAL = 0x080, LORENTZMATERIAL = 0x100,
        DEBYEMATERIAL = 0x200, DISCRETE_MATERIAL = 0x400, LUMPED_ELEMENT = 0x800, CONDUCTINGSHEET = 0x1000
    };
    virtual ~CSProperties() {}
};

class ContinuousStructure {
public:
    virtual ~ContinuousStructure() {}
};
