{
   /* Point lights and omni emitters: an omni point light, an oriented point light, an omni
    * unit plane hanging vertically (emits on both faces) and an omni OBJ mesh, in an open box. */
   "scenefile" : {
      "renderer" : { "type" : "pathTracer", "noSuperSamples" : 16, "noDirectSamples" : 4,
                     "maxDepth" : 5, "rrStartDepth" : 3, },
      "camera" : { "type" : "pinhole", "eye" : [ 0, 1, 3.4 ], "look" : [ 0, -0.1, -1 ], "up" : [ 0, 1, 0 ],
                   "heightAngle" : 45, },
      "output" : { "width" : 40, "height" : 40, },
      "scene" : {
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.7, 0.7, 0.7 ], },
            "plane" : { "vertices" : [ -1.5, 0, 1.5,   1.5, 0, 1.5,   1.5, 0, -1.5,   -1.5, 0, -1.5 ], },
            "plane" : { "vertices" : [ -1.5, 0, -1.5,   1.5, 0, -1.5,   1.5, 2.5, -1.5,   -1.5, 2.5, -1.5 ], },
         },
         "material" : {
            "bsdf" : { "type" : "phong", "kd" : 0.3, "ks" : 0.4, "n" : 30, },
            "transform" : { "translate" : [ 0.6, 0.35, -0.3 ], "scale" : [ 0.7, 0.7, 0.7 ], "cube" : { }, },
         },
         "material" : {
            "emitter" : { "type" : "omni", "power" : [ 24, 20, 16 ], },
            "transform" : { "translate" : [ -0.5, 1.6, 0.2 ], "point" : { }, },
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 3, 5, 8 ], },
            "transform" : { "translate" : [ 0.9, 1.2, 0.8 ], "point" : { }, },
         },
         "material" : {
            "emitter" : { "type" : "omni", "power" : [ 2, 0.5, 0.5 ], },
            "bsdf" : { "type" : "diffuse", "kd" : 0.2, },
            "transform" : {
               "translate" : [ -0.9, 0.6, -0.6 ],
               "rotate" : [ 0, 0, 0,  0, 0, 1,  90 ],
               "scale" : [ 0.5, 1, 0.5 ],
               "plane" : { },
            },
         },
         "material" : {
            "emitter" : { "type" : "omni", "power" : [ 0.4, 1.5, 0.6 ], },
            "bsdf" : { "type" : "diffuse", "kd" : 0.3, },
            "transform" : {
               "translate" : [ -0.1, 0.25, 0.6 ],
               "scale" : [ 0.2, 0.2, 0.2 ],
               "mesh" : { "path" : "octahedron.obj", },
            },
         },
      },
   },
}
