{
   /* A closed box lit by one unit-plane emitter, written for the loader tests:
    * materials, a transformed unit plane light, planes given by vertices, a cube and a mesh. */
   "scenefile" : {
      "version" : 0.1,
      "renderer" : {
         "type" : "pathTracer",
         "noSuperSamples" : 16,
         "noDirectSamples" : 1,
         "maxDepth" : 5,
         "rrStartDepth" : 3,
      },
      "camera" : {
         "type" : "pinhole",
         "eye" : [ 0, 1, 3.5 ],
         "look" : [ 0, 0, -1 ],
         "up" : [ 0, 1, 0 ],
         "heightAngle" : 40,
      },
      "output" : { "width" : 48, "height" : 40, },
      "scene" : {
         "triangle" : { /* default material, listed first but flattened after every material */
            "vertices" : [ -0.2, 0.01, 0.5,   0.2, 0.01, 0.5,   0.0, 0.01, 0.2 ],
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 12, 12, 10 ], },
            "bsdf" : { "type" : "diffuse", "kd" : 0, },
            "transform" : {
               "translate" : [ 0, 1.99, 0 ],
               "rotate" : [ 0, 0, 0,  1, 0, 0,  180 ],
               "scale" : [ 0.5, 1, 0.5 ],
               "plane" : { },
            },
         },
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.7, 0.7, 0.6 ], },
            "plane" : { "vertices" : [ -1, 0, 1,   1, 0, 1,   1, 0, -1,   -1, 0, -1 ], },
            "plane" : { "vertices" : [ -1, 2, -1,   1, 2, -1,   1, 2, 1,   -1, 2, 1 ], },
            "plane" : { "vertices" : [ -1, 0, -1,   1, 0, -1,   1, 2, -1,   -1, 2, -1 ], },
         },
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.6, 0.2, 0.2 ], },
            "plane" : { "vertices" : [ -1, 0, 1,   -1, 0, -1,   -1, 2, -1,   -1, 2, 1 ], },
         },
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.2, 0.6, 0.2 ], },
            "plane" : { "vertices" : [ 1, 0, -1,   1, 0, 1,   1, 2, 1,   1, 2, -1 ], },
         },
         "material" : {
            "bsdf" : { "type" : "phong", "kd" : 0.3, "ks" : 0.5, "n" : 40, },
            "transform" : {
               "translate" : [ -0.35, 0.45, -0.3 ],
               "rotate" : [ 0, 0, 0,  0, 1, 0,  25 ],
               "scale" : [ 0.5, 0.9, 0.5 ],
               "cube" : { },
            },
         },
         "material" : {
            "bsdf" : { "type" : "dielectric", "ior" : 1.5, },
            "transform" : {
               "translate" : [ 0.4, 0.3, 0.3 ],
               "scale" : [ 0.3, 0.3, 0.3 ],
               "mesh" : { "path" : "octahedron.obj", },
            },
         },
      },
   },
}
